"""Writes the basis-set files this package ships, from a Basis Set Exchange JSON directory.

    python make_basis_sets.py <bse_json_dir>

Keeps the BSE JSON schema the reference program reads (its basis_sets/ directory), trimmed to the
elements H-Ne and to the fields the reader uses (elements -> electron_shells -> angular_momentum,
exponents, coefficients).  Values are copied as the original strings.
"""
import json
import os
import sys

NAMES = ["sto-3g", "sto-6g", "6-31g", "6-31g_st__st_", "6-311g_st_", "6-311g_st__st_", "cc-pvdz"]


def main(src: str) -> None:
    here = os.path.dirname(os.path.abspath(__file__))
    for name in NAMES:
        path = os.path.join(src, name + ".json")
        if not os.path.exists(path):
            continue
        with open(path) as f:
            data = json.load(f)
        out = {"name": data.get("name", name), "elements": {}}
        for z, el in data["elements"].items():
            if 1 <= int(z) <= 10:
                out["elements"][z] = {"electron_shells": [
                    {k: sh[k] for k in ("angular_momentum", "exponents", "coefficients")}
                    for sh in el["electron_shells"]]}
        with open(os.path.join(here, name + ".json"), "w") as f:
            json.dump(out, f, indent=1)
        print("wrote", name)


if __name__ == "__main__":
    main(sys.argv[1])
