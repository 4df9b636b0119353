"""Golden fixtures at the benchmarked sizes, generated from the reference program itself (needs oracle/_ref).

    python tests/golden/make_golden_configs.py w16 [fd_w8]

* ``cfg_w16_631gss``: (H2O)_16 on a 4x2x2 lattice (seed 0), RHF/6-31G** (192 shells, 400 basis functions).
  The reference's basis structure of arrays, its Schwartz matrix Q, the core-guess density Da, the full
  direct Fock build on it (F = J - K), the converged SCF density Da_scf and energy (ENERGY_TOL 1e-10), and
  the incremental build from the guess to the converged density (F_inc = F + J[dD] - K[dD],
  SCF.cpp:731-743).  The wall time of the reference's full Fock build is recorded as well
  (``ref_fock_s``, ``ref_threads``), for the calibration of the C restatement against it.
* ``cfg_fd_w8_ccpvdz``: (H2O)_8 on a 2x2x2 lattice, RHF/cc-pVDZ (144 basis functions under the reference's
  basis reader).  Central differences (+-1e-4 bohr) of the reference's total energy for nine Cartesian
  coordinates (``coords``: atom, axis) -- the three axes of three atoms in different waters.  One
  reference SCF at this size takes ~4.5 minutes on 8 cores, so the full 72-coordinate gradient (145
  SCFs) is out of reach; the analytic gradient's other components are covered by translational
  invariance and the smaller FD fixtures.  Same tight settings as make_fd_gradients.py.
"""
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, REPO)
sys.path.insert(0, os.path.join(REPO, "hartree-fock_gb300"))

from hfgpu import workloads as w  # noqa: E402
from oracle import ref  # noqa: E402

SCF_TIGHT = dict(ENERGY_TOL="1e-10", DENSITY_TOL="1e-7", DIIS_TOL="1e-7", MAX_ITER=100)
FD_TIGHT = dict(ENERGY_TOL="1e-11", DENSITY_TOL="1e-9", DIIS_TOL="1e-9", MAX_ITER=300, SCHWARTZ_THRESH="1e-14",
                DENSITY_THRESH="1e-14")
FD_STEP = 1e-4
# (atom, axis): O of water 0, H of water 3, O of water 7 (atom order per water: H, H, O).
FD_COORDS = [(2, 0), (2, 1), (2, 2), (10, 0), (10, 1), (10, 2), (23, 0), (23, 1), (23, 2)]


def make_w16():
    Z, xyz = w.water_lattice(4, 2, 2)
    kw = dict(w.BENCH_SCF)
    kw.update(SCF_TIGHT)
    text = w.input_text(Z, xyz, "6-31G**", **kw)
    s = ref.RefSession(text)
    soa = s.basis_soa()
    Q = s.schwartz()
    Da, Db = s.guess()
    t0 = time.perf_counter()
    Fa, Fb = s.fock_direct(Da, Db)
    ref_fock_s = time.perf_counter() - t0
    t0 = time.perf_counter()
    r = s.scf_run()
    ref_scf_s = time.perf_counter() - t0
    Da_scf = r["Da"]
    Fa_inc, _ = s.fock_direct(Da_scf, r["Db"], Da, Db, Fa, Fb)
    e_total = r["e_elec"] + r["e_nuc"]
    out = dict(input_text=np.array(text), Z=np.array(Z, np.int32), xyz=np.array(xyz), basis=np.array("6-31G**"),
               charge=0, multiplicity=1, unrestricted=0, nocc_a=s.nocc_a, nocc_b=s.nocc_b,
               nuclear_repulsion=s.nuclear_repulsion, Q=Q, Da=Da, Fa=Fa, Da_scf=Da_scf, Fa_inc=Fa_inc,
               e_elec=r["e_elec"], e_nuc=r["e_nuc"], e_total=e_total, scf_iterations=r["iterations"],
               ref_fock_s=ref_fock_s, ref_scf_s=ref_scf_s, ref_threads=os.cpu_count(),
               **{"soa_" + k: v for k, v in soa.items()})
    np.savez_compressed(os.path.join(HERE, "cfg_w16_631gss.npz"), **out)
    print(f"cfg_w16_631gss: E_total {e_total:.10f} in {r['iterations']} iterations; reference full Fock build "
          f"{ref_fock_s:.2f} s, SCF {ref_scf_s:.1f} s on {os.cpu_count()} threads")


def fd_energy(Z, xyz):
    kw = dict(w.BENCH_SCF)
    kw.update(FD_TIGHT)
    s = ref.RefSession(w.input_text(Z, xyz, "cc-pVDZ", **kw))
    r = s.scf_run()
    s.close()
    return r["e_elec"] + r["e_nuc"]


def make_fd_w8():
    Z, xyz0 = w.water_lattice(2, 2, 2)
    path = os.path.join(HERE, "cfg_fd_w8_ccpvdz.npz")
    g = np.full(len(FD_COORDS), np.nan)
    if os.path.exists(path):  # resume: keep the coordinates already done
        g = np.array(np.load(path)["grad_fd"], dtype=float)
    for k, (a, ax) in enumerate(FD_COORDS):
        if not np.isnan(g[k]):
            continue
        xp, xm = xyz0.copy(), xyz0.copy()
        xp[a, ax] += FD_STEP
        xm[a, ax] -= FD_STEP
        g[k] = (fd_energy(Z, xp) - fd_energy(Z, xm)) / (2 * FD_STEP)
        print(f"cfg_fd_w8_ccpvdz: atom {a} axis {ax} dE/dx = {g[k]:.9f}", flush=True)
        # Written after every coordinate, so that an interrupted run keeps what it has (NaN = not yet).
        np.savez_compressed(path, Z=np.array(Z, np.int32), xyz=xyz0, basis=np.array("cc-pVDZ"), charge=0,
                            multiplicity=1, coords=np.array(FD_COORDS, np.int32), grad_fd=g, step=FD_STEP,
                            threshold=1e-14, extra=np.array("{}"))


if __name__ == "__main__":
    for name in sys.argv[1:] or ["w16", "fd_w8"]:
        {"w16": make_w16, "fd_w8": make_fd_w8}[name]()
