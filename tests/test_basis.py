"""Basis packing (hfgpu.basis) against the reference's IntegralEngine arrays (golden fixtures)."""
import numpy as np
import pytest

from conftest import GOLDEN_NAMES, load_golden


@pytest.mark.parametrize("name", GOLDEN_NAMES)
def test_pack_matches_reference_soa(name):
    from hfgpu import basis

    g = load_golden(name)
    soa = basis.pack(str(g["basis"]), g["Z"], g["xyz"])
    for k, ref in g["soa"].items():
        got = np.asarray(soa[k])
        assert got.shape == ref.shape, k
        if ref.dtype.kind == "i":
            assert np.array_equal(got, ref), k
        else:
            assert np.max(np.abs(got - ref)) <= 1e-15 * max(1.0, np.abs(ref).max()), k


def test_unknown_basis_raises():
    from hfgpu import basis

    with pytest.raises(FileNotFoundError):
        basis.pack("no-such-basis", [1], [[0, 0, 0]])


def test_workload_coordinates_roundtrip_through_input_text():
    from hfgpu import workloads as w

    Z, x = w.water_lattice(2, 2, 1)
    text = w.input_text(Z, x, "6-31G")
    rows = [l.split() for l in text.splitlines() if l.strip()[:1] in ("H", "O")]
    parsed = np.array([[float(v) for v in r[1:4]] for r in rows])
    assert np.array_equal(parsed, x)


def test_general_contractions_opt_in():
    """Opt-in extension: one shell per coefficient row of a generally contracted shell (cc-pVDZ); the
    default keeps the reference's first-row rule, and segmented sets (6-31G**) are unchanged."""
    from hfgpu import basis, workloads

    Z, xyz = workloads.monomer()
    ref = basis.pack("cc-pVDZ", Z, xyz)
    gen = basis.pack("cc-pVDZ", Z, xyz, general_contractions=True)
    nbf = lambda s: int(sum((l + 1) * (l + 2) // 2 for l in s["l"]))
    assert nbf(ref) == 18 and nbf(gen) == 25  # O 3s2p1d + H 2s1p each, Cartesian d
    assert np.all(gen["coeff"] != 0.0)
    seg = basis.pack("6-31G**", Z, xyz, general_contractions=True)
    seg0 = basis.pack("6-31G**", Z, xyz)
    assert all(np.array_equal(seg[k], seg0[k]) for k in seg)
