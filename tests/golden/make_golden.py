"""Generates the golden fixtures of tests/golden from the reference program itself.

    python tests/golden/make_golden.py            (needs oracle/_ref, built by oracle/Makefile.ref)

For each small system: the reference's basis structure of arrays, Schwartz matrix Q, core-guess
densities, one full direct Fock build on the guess (F = J - K with F_prev = 0, SCF.cpp:523-744), one
incremental build on a perturbed density, the one-electron matrices, and the converged SCF energy
(SCF::run).  Stored as compressed .npz, a few hundred KB in total.
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

TIGHT = dict(ENERGY_TOL="1e-10", DENSITY_TOL="1e-7", DIIS_TOL="1e-7", MAX_ITER=100)

SYSTEMS = {
    # The water monomer, RHF/6-31G, DIIS size 6 (the smallest benchmarked case).
    "h2o_631g": (w.monomer, "6-31G", 0, 1, dict(DIIS_SIZE=6)),
    # The reference README example: UHF with HOMO/LUMO mixing, here on the +1 doublet.
    "h2o_cation_uhf_631g": (w.monomer, "6-31G", 1, 2, dict(UNRESTRICTED=True, GUESS_MIX=2)),
    "w2_631gss": (lambda: w.water_lattice(2, 1, 1), "6-31G**", 0, 1, {}),
    "w2_ccpvdz": (lambda: w.water_lattice(2, 1, 1), "cc-pVDZ", 0, 1, {}),
    "w4_631gss": (lambda: w.water_lattice(2, 2, 1), "6-31G**", 0, 1, {}),
    "w2_cation_uhf_631gss": (lambda: w.water_lattice(2, 1, 1), "6-31G**", 1, 2, dict(GUESS_MIX=2)),
    # The stored-integral SCF (DIRECT FALSE: SCF::buildFockMatrix from electronRepulsionTensor).
    "h2o_631g_conv": (w.monomer, "6-31G", 0, 1, dict(DIRECT=False)),
    "w2_ccpvdz_conv": (lambda: w.water_lattice(2, 1, 1), "cc-pVDZ", 0, 1, dict(DIRECT=False)),
}


def make(name, spec, run_scf=True):
    geo, basis, charge, mult, extra = spec
    Z, xyz = geo()
    kw = dict(w.BENCH_SCF)
    kw.update(TIGHT)
    kw.update(extra)
    text = w.input_text(Z, xyz, basis, charge=charge, multiplicity=mult, **kw)
    s = ref.RefSession(text.replace("DIRECT             FALSE", "DIRECT             TRUE"))
    soa = s.basis_soa()
    Q = s.schwartz()
    Da, Db = s.guess()
    Fa, Fb = s.fock_direct(Da, Db)
    rng = np.random.default_rng(7)
    P = 1e-3 * rng.standard_normal(Da.shape)
    P = P + P.T
    Da2, Db2 = Da + P, Db + (P if s.unrestricted else P)
    Fa2, Fb2 = s.fock_direct(Da2, Db2, Da, Db, Fa, Fb)
    S, T, V = s.one_electron()
    out = dict(input_text=np.array(text), Z=np.array(Z, np.int32), xyz=np.array(xyz), basis=np.array(basis),
               charge=charge, multiplicity=mult, unrestricted=int(s.unrestricted), nocc_a=s.nocc_a, nocc_b=s.nocc_b,
               nuclear_repulsion=s.nuclear_repulsion, Q=Q, Da=Da, Db=Db, Fa=Fa, Fb=Fb, Da2=Da2, Db2=Db2, Fa2=Fa2,
               Fb2=Fb2, S=S, T=T, V=V, **{"soa_" + k: v for k, v in soa.items()})
    if run_scf:
        if extra.get("DIRECT", True) is False:
            # The reference's direct-build entry points need the direct set-up: the matrices above come
            # from a DIRECT TRUE session of the same input; the SCF runs with the stored integrals.
            s.close()
            s = ref.RefSession(text)
        r = s.scf_run()
        out.update(e_elec=r["e_elec"], e_nuc=r["e_nuc"], scf_iterations=r["iterations"], Da_scf=r["Da"],
                   Db_scf=r["Db"])
        print(name, "E_total", r["e_elec"] + r["e_nuc"], "iterations", r["iterations"])
    np.savez_compressed(os.path.join(HERE, name + ".npz"), **out)


if __name__ == "__main__":
    names = sys.argv[1:] or list(SYSTEMS)
    for n in names:
        make(n, SYSTEMS[n])
