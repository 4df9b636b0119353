"""GPU parity of the direct Fock build against the reference (golden fixtures) and the CPU oracle.

Tolerances: FP64 path -- Fock matrices within 1e-10 Eh max-abs of the reference; quartet survival lists
bit-identical given the reference's Schwartz matrix.  Mixed path -- within 1e-6 of the FP64 result on
these small systems (the per-quartet FP32 error bound is fp32_cutoff * 1e-6 relative).
"""
import numpy as np
import pytest

from conftest import GOLDEN_NAMES, load_golden

pytestmark = pytest.mark.gpu


def engine_for(g):
    from hfgpu.engine import Engine

    return Engine(g["soa"])


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_gpu_schwartz_matches_reference(name):
    g = load_golden(name)
    e = engine_for(g)
    Q = e.schwartz()
    assert np.max(np.abs(Q - g["Q"])) <= 1e-12 * max(1.0, np.abs(g["Q"]).max())


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_gpu_fock_fp64_matches_reference(name):
    g = load_golden(name)
    e = engine_for(g)
    e.set_schwartz(g["Q"])
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J, Ka, Kb, st = e.fock(Da + Db, Da, Db if uhf else None)
    assert np.max(np.abs((J - Ka) - g["Fa"])) <= 1e-10
    if uhf:
        assert np.max(np.abs((J - Kb) - g["Fb"])) <= 1e-10
    assert np.allclose(J, J.T, atol=0) and np.allclose(Ka, Ka.T, atol=0)
    # Incremental build, F = F_prev + J[dD] - K[dD] (SCF.cpp:731-743).
    dA, dB = g["Da2"] - Da, g["Db2"] - Db
    J2, Ka2, Kb2, _ = e.fock((g["Da2"] + g["Db2"]) - (Da + Db), dA, dB if uhf else None)
    assert np.max(np.abs(g["Fa"] + J2 - Ka2 - g["Fa2"])) <= 1e-10
    if uhf:
        assert np.max(np.abs(g["Fb"] + J2 - Kb2 - g["Fb2"])) <= 1e-10


@pytest.mark.parametrize("name", ["h2o_631g", "w2_631gss", "w4_631gss", "h2o_cation_uhf_631g"])
def test_gpu_survivors_bit_identical(port, name):
    g = load_golden(name)
    e = engine_for(g)
    e.set_schwartz(g["Q"])
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    rng = np.random.default_rng(11)
    # A density increment with many tiny entries so that the density predicate matters.
    P = rng.standard_normal(Da.shape) * 10.0 ** rng.uniform(-14, -6, Da.shape)
    P = P + P.T
    e.fock(2 * P, P, P if uhf else None)
    got = e.survivors()
    B = port.Basis(g["soa"])
    want = B.survivors(g["Q"], 2 * P, P, P if uhf else None)
    assert got.shape == want.shape
    assert np.array_equal(got, want)


@pytest.mark.parametrize("name", ["w2_631gss", "w2_ccpvdz"])
def test_gpu_eri_blocks_match_oracle(port, name):
    g = load_golden(name)
    e = engine_for(g)
    B = port.Basis(g["soa"])
    ns = B.nshells
    rng = np.random.default_rng(5)
    for _ in range(60):
        a, b, c, d = (int(x) for x in rng.integers(0, ns, 4))
        got = e.eri_block(a, b, c, d)
        # The oracle's block carries the reference's zero pattern; compare where it is defined.
        want = B.eri(max(a, b), min(a, b), max(c, d), min(c, d))
        gotc = e.eri_block(max(a, b), min(a, b), max(c, d), min(c, d))
        mask = want != 0
        assert np.max(np.abs(gotc[mask] - want[mask])) <= 1e-12 * max(1.0, np.abs(want).max())
        assert got.shape == tuple(B.nao_of(s) for s in (a, b, c, d))


@pytest.mark.parametrize("name", ["w2_631gss", "w4_631gss", "w2_cation_uhf_631gss"])
def test_gpu_mixed_precision_close_to_fp64(name):
    g = load_golden(name)
    e = engine_for(g)
    uhf = bool(g["unrestricted"])
    Da, Db = g["Da"], g["Db"]
    J64, K64, Kb64, s64 = e.fock(Da + Db, Da, Db if uhf else None)
    J32, K32, Kb32, s32 = e.fock(Da + Db, Da, Db if uhf else None, precision=1, fp32_cutoff=1e-4)
    assert sum(s32["quartets_fp32"]) > 0
    assert sum(s32["quartets_fp32"]) + sum(s32["quartets_fp64"]) == sum(s64["quartets_fp64"])
    assert np.max(np.abs(J32 - J64)) <= 1e-6
    assert np.max(np.abs(K32 - K64)) <= 1e-6


def test_gpu_batch_equals_single_molecules():
    from hfgpu.engine import Engine

    gs = [load_golden(n) for n in ("h2o_631g", "w2_631gss", "w2_ccpvdz")]
    eb = Engine([g["soa"] for g in gs])
    dt = np.concatenate([(2 * g["Da"]).ravel(order="F") for g in gs])
    da = np.concatenate([g["Da"].ravel(order="F") for g in gs])
    J, K, _, _ = eb.fock(dt, da)
    off = 0
    for g in gs:
        n = g["Da"].shape[0]
        e1 = Engine(g["soa"])
        J1, K1, _, _ = e1.fock(2 * g["Da"], g["Da"])
        Jb = J[off:off + n * n].reshape(n, n, order="F")
        Kb = K[off:off + n * n].reshape(n, n, order="F")
        assert np.max(np.abs(Jb - J1)) <= 1e-12 and np.max(np.abs(Kb - K1)) <= 1e-12
        off += n * n


def test_gpu_fock_into_caller_buffers():
    from hfgpu.engine import Engine

    g = load_golden("w2_631gss")
    e = Engine(g["soa"])
    Da = g["Da"]
    J, K, _, _ = e.fock(2 * Da, Da)
    out = [np.full(Da.size, np.nan), np.full(Da.size, np.nan)]
    J2, K2, _, _ = e.fock(2 * Da, Da, out=out)
    assert np.shares_memory(J2, out[0]) and np.shares_memory(K2, out[1])
    assert np.max(np.abs(J2 - J)) <= 1e-12 and np.max(np.abs(K2 - K)) <= 1e-12
    with pytest.raises(ValueError):
        e.fock(2 * Da, Da, out=[np.zeros(3), np.zeros(3)])
