"""Seeded synthetic water-cluster workloads and reference-format input files.

The reference program reads a ``$molecule / $scf / $basis`` input (src/Input.cpp:23-146; format in the
reference README, "Input File Example").  These helpers write exactly that format, for the systems the
benchmarks are quoted on:

* the water monomer of the reference README example (geometry in bohr, atoms H, H, O);
* ``(H2O)_n`` lattices: each copy of the monomer is rotated about its centroid by a unit quaternion
  ``q = n/|n|`` with ``n ~ N(0,1)^4``, moved so that its centroid sits on the lattice point, and shifted
  by a jitter ``U(-0.2, 0.2)`` bohr per axis;
* 1-D chains of ``k`` rotated waters with 5.5 bohr spacing (no jitter), for batches of uneven molecules.

All randomness comes from ``numpy.random.default_rng(seed)``; the draw order is fixed (per molecule: the
four quaternion normals, then the three jitters) so a seed names one geometry.
"""
from __future__ import annotations

import numpy as np

# Water monomer, bohr, atom order H, H, O (reference README, "Input File Example").
WATER_Z = (1, 1, 8)
WATER_XYZ = np.array(
    [
        [1.4327076887, -0.9610871670, 0.0],
        [-1.4327076887, -0.9610871670, 0.0],
        [0.0, 0.2403536480, 0.0],
    ]
)
SYMBOLS = {1: "H", 2: "He", 3: "Li", 4: "Be", 5: "B", 6: "C", 7: "N", 8: "O", 9: "F", 10: "Ne"}


def quaternion_rotation(n: np.ndarray) -> np.ndarray:
    """3x3 rotation matrix of the unit quaternion n/|n| (n = (w, x, y, z))."""
    w, x, y, z = n / np.linalg.norm(n)
    return np.array(
        [
            [1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)],
            [2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)],
            [2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)],
        ]
    )


def _as_written(x: np.ndarray) -> np.ndarray:
    """Coordinates exactly as the input file states them (10 decimals, parsed back)."""
    return np.vectorize(lambda v: float(f"{v:.10f}"))(x)


def _place(rng: np.random.Generator, point: np.ndarray, jitter: float) -> np.ndarray:
    centroid = WATER_XYZ.mean(axis=0)
    rot = quaternion_rotation(rng.standard_normal(4))
    shift = rng.uniform(-jitter, jitter, 3) if jitter > 0 else np.zeros(3)
    return _as_written((WATER_XYZ - centroid) @ rot.T + point + shift)


def water_lattice(nx: int, ny: int, nz: int, spacing: float = 5.5, seed: int = 0, jitter: float = 0.2):
    """(H2O)_{nx*ny*nz} on a lattice; returns (Z list, coords (natom,3) bohr)."""
    rng = np.random.default_rng(seed)
    Z, xyz = [], []
    for i in range(nx):
        for j in range(ny):
            for k in range(nz):
                xyz.append(_place(rng, np.array([i, j, k], float) * spacing, jitter))
                Z.extend(WATER_Z)
    return Z, np.concatenate(xyz, axis=0)


def water_chain(k: int, rng: np.random.Generator, spacing: float = 5.5):
    """A 1-D chain of k rotated waters along x (no jitter)."""
    Z, xyz = [], []
    for i in range(k):
        xyz.append(_place(rng, np.array([i * spacing, 0.0, 0.0]), 0.0))
        Z.extend(WATER_Z)
    return Z, np.concatenate(xyz, axis=0)


def uneven_batch(count: int = 256, kmax: int = 12, seed: int = 0):
    """``count`` chains (H2O)_k with k ~ U{1..kmax}; returns a list of (Z, coords)."""
    rng = np.random.default_rng(seed)
    sizes = rng.integers(1, kmax + 1, size=count)
    return [water_chain(int(k), rng) for k in sizes]


def monomer():
    return list(WATER_Z), WATER_XYZ.copy()


def input_text(Z, xyz, basis: str, charge: int = 0, multiplicity: int = 1, **scf) -> str:
    """Reference-format input.  ``scf`` maps $scf keywords (case-insensitive) to values."""
    lines = ["$molecule", f"    {charge}    {multiplicity}"]
    for z, (x, y, zz) in zip(Z, xyz):
        lines.append(f"    {SYMBOLS[int(z)]:<2} {x: .10f} {y: .10f} {zz: .10f}")
    lines.append("$end")
    lines.append("$scf")
    for key, val in scf.items():
        if isinstance(val, bool):
            val = "TRUE" if val else "FALSE"
        lines.append(f"    {key.upper():<18} {val}")
    lines.append("$end")
    lines += ["$basis", f"    {basis}", "$end", ""]
    return "\n".join(lines)


# Keywords shared by every generated benchmark input: direct SCF, no reorientation, 1e-10 screening.
BENCH_SCF = dict(SYMMETRY=False, DIRECT=True, SCHWARTZ_THRESH="1e-10", DENSITY_THRESH="1e-10")
