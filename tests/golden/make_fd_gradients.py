"""Central finite-difference nuclear gradients of the reference program's SCF energy (golden fixtures
for the analytic-gradient tests): E(x +- 1e-4 bohr) for every Cartesian coordinate, each SCF converged
tightly (ENERGY_TOL 1e-11, DENSITY_TOL 1e-9, DIIS_TOL 1e-9) with SCHWARTZ_THRESH = DENSITY_THRESH = 1e-14:
at the default 1e-10 the incremental builds leave a ~5e-8 Eh noise floor that the 2e-4 bohr difference
would amplify.  Needs oracle/_ref.

    python tests/golden/make_fd_gradients.py [name ...]
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "hartree-fock_gb300"))

from hfgpu import workloads as w  # noqa: E402
from oracle import ref  # noqa: E402

STEP = 1e-4
TIGHT = dict(ENERGY_TOL="1e-11", DENSITY_TOL="1e-9", DIIS_TOL="1e-9", MAX_ITER=300, SCHWARTZ_THRESH="1e-14",
             DENSITY_THRESH="1e-14")
SYSTEMS = {
    "fd_h2o_631g": (w.monomer, "6-31G", 0, 1, {}),
    "fd_h2o_cation_uhf_631g": (w.monomer, "6-31G", 1, 2, dict(GUESS_MIX=2)),
    "fd_w2_631gss": (lambda: w.water_lattice(2, 1, 1), "6-31G**", 0, 1, {}),
    "fd_h2o_ccpvdz": (w.monomer, "cc-pVDZ", 0, 1, {}),
}


def energy(Z, xyz, basis, charge, mult, extra):
    kw = dict(w.BENCH_SCF)
    kw.update(TIGHT)  # overrides the 1e-10 screening thresholds
    kw.update(extra)
    s = ref.RefSession(w.input_text(Z, xyz, basis, charge=charge, multiplicity=mult, **kw))
    r = s.scf_run()
    s.close()
    return r["e_elec"] + r["e_nuc"]


def make(name):
    geo, basis, charge, mult, extra = SYSTEMS[name]
    Z, xyz0 = geo()
    g = np.zeros_like(xyz0)
    e0 = energy(Z, xyz0, basis, charge, mult, extra)
    for a in range(len(Z)):
        for k in range(3):
            xp, xm = xyz0.copy(), xyz0.copy()
            xp[a, k] += STEP
            xm[a, k] -= STEP
            g[a, k] = (energy(Z, xp, basis, charge, mult, extra) - energy(Z, xm, basis, charge, mult, extra)) / (2 * STEP)
    np.savez_compressed(os.path.join(HERE, name + ".npz"), Z=np.array(Z, np.int32), xyz=xyz0, basis=np.array(basis),
                        charge=charge, multiplicity=mult, energy=e0, grad_fd=g, step=STEP, threshold=1e-14,
                        extra=np.array(repr(extra)))
    print(name, "E", e0, "max|g|", np.abs(g).max(), "sum g", g.sum(axis=0))


if __name__ == "__main__":
    for n in sys.argv[1:] or list(SYSTEMS):
        make(n)
