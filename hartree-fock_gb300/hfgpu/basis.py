"""Basis-set reading and packing into the engine's structure of arrays (test and benchmark helper).

Follows the reference's rules exactly (src/Basis.cpp):
* file ``basis_sets/<name>.json`` with the name lower-cased and every ``*`` replaced by ``_st_``
  (Basis.cpp:91-104), Basis Set Exchange JSON schema;
* for each element shell and each entry ``i`` of its ``angular_momentum`` list, one shell of that
  angular momentum with all exponents and the ``i``-th coefficient row only (Basis.cpp:125-159) -- so a
  generally contracted shell keeps its first contraction only;
* shells in atom order, per atom in file order (Basis.cpp:25-84);
* Cartesian components with the x exponent descending, then y descending (Basis.cpp:48-59);
* per primitive and component the factor (2a/pi)^{3/4} (4a)^{l/2} / sqrt((2i-1)!!(2j-1)!!(2k-1)!!)
  (Basis.cpp:61-77); contraction coefficients are not renormalised.

Opt-in extension (``general_contractions=True``; changes the numbers against the reference): a generally
contracted shell -- one angular momentum with several coefficient rows, e.g. the s and p shells of the
cc-pVXZ sets -- becomes one shell per coefficient row, each holding the exponents whose coefficient in
that row is non-zero.  Shells that list several angular momenta (the Pople sp shells) keep the reference
rule of one row per angular momentum.
"""
from __future__ import annotations

import json
import math
import os

import numpy as np

DEFAULT_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "basis_sets")


def basis_file(name: str, directory: str | None = None) -> str:
    return os.path.join(directory or DEFAULT_DIR, name.lower().replace("*", "_st_") + ".json")


def _dfact(n: int) -> int:
    r = 1
    while n > 1:
        r *= n
        n -= 2
    return r


def cart_components(l: int):
    return [(i, j, l - i - j) for i in range(l, -1, -1) for j in range(l - i, -1, -1)]


def read_shells(name: str, elements, directory: str | None = None, general_contractions: bool = False):
    """{Z: [(l, exponents, coefficients), ...]} for the requested elements."""
    path = basis_file(name, directory)
    if not os.path.exists(path):
        raise FileNotFoundError(f"Basis set '{name}' not found.")
    with open(path) as f:
        data = json.load(f)
    out = {}
    for Z in sorted(set(int(z) for z in elements)):
        el = data["elements"].get(str(Z))
        if el is None:
            raise KeyError(f"element {Z} not found in basis set '{name}'.")
        shells = []
        for sh in el["electron_shells"]:
            exps = [float(x) for x in sh["exponents"]]
            ams = sh["angular_momentum"]
            if general_contractions and len(ams) == 1 and len(sh["coefficients"]) > 1:
                for row in sh["coefficients"]:
                    keep = [(a, float(c)) for a, c in zip(exps, row) if float(c) != 0.0]
                    shells.append((int(ams[0]), [a for a, _ in keep], [c for _, c in keep]))
                continue
            for i, l in enumerate(ams):
                coefs = [float(x) for x in sh["coefficients"][i]]
                shells.append((int(l), exps, coefs))
        out[Z] = shells
    return out


def pack(name: str, Z, xyz, directory: str | None = None, general_contractions: bool = False) -> dict:
    """The engine's SoA for a molecule (atoms Z at xyz, bohr); see the module notes for the opt-in
    ``general_contractions``."""
    table = read_shells(name, Z, directory, general_contractions)
    l_, nprim, prim_off, ao_off, norm_off, centers = [], [], [], [], [], []
    alpha, coeff, norms, am = [], [], [], []
    po = ao = no = 0
    for z, r in zip(Z, np.asarray(xyz, float)):
        for (l, exps, coefs) in table[int(z)]:
            comps = cart_components(l)
            l_.append(l)
            nprim.append(len(exps))
            prim_off.append(po)
            ao_off.append(ao)
            norm_off.append(no)
            centers.append(r)
            alpha += exps
            coeff += coefs[: len(exps)]
            for a in exps:
                for (i, j, k) in comps:
                    norms.append((2 * a / math.pi) ** 0.75 * (4 * a) ** ((i + j + k) / 2.0)
                                 / math.sqrt(_dfact(2 * i - 1) * _dfact(2 * j - 1) * _dfact(2 * k - 1)))
            am += comps
            po += len(exps)
            ao += len(comps)
            no += len(exps) * len(comps)
    return dict(l=np.array(l_, np.int32), nprim=np.array(nprim, np.int32), prim_off=np.array(prim_off, np.int32),
                ao_off=np.array(ao_off, np.int32), norm_off=np.array(norm_off, np.int32),
                centers=np.array(centers, float).reshape(-1, 3), alpha=np.array(alpha), coeff=np.array(coeff),
                norms=np.array(norms), am=np.array(am, np.int32).reshape(-1, 3))
