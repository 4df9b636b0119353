"""Calibration of the plain-C restatement (oracle/hf_oracle.c, built with the reference's release flags)
against the reference program itself (oracle/_ref, its own sources and flags) on the same host: one full
direct Fock build of (H2O)_16 RHF/6-31G** (400 basis functions, the seeded 4x2x2 lattice) on the
reference's core-guess density, with the reference's Schwartz matrix, through each of them, with the same
OpenMP thread count.  Prints one JSON line: both wall times, their ratio, and the largest difference of
the two Fock matrices.

Test infrastructure: it needs oracle/_ref, which is built only where the reference's sources are present.

    python oracle/calibrate.py [repeats]
"""
import json
import os
import sys
import time

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.join(os.path.dirname(HERE), "hartree-fock_gb300"))

import numpy as np  # noqa: E402

from hfgpu import workloads as w  # noqa: E402
from oracle import port, ref  # noqa: E402


def main():
    repeats = int(sys.argv[1]) if len(sys.argv) > 1 else 2
    Z, xyz = w.water_lattice(4, 2, 2)
    s = ref.RefSession(w.input_text(Z, xyz, "6-31G**", **w.BENCH_SCF))
    Q = s.schwartz()
    Da, Db = s.guess()
    B = port.Basis(s.basis_soa(), release=True)
    t_ref, t_port = [], []
    for _ in range(repeats):
        t0 = time.perf_counter()
        Fa, _ = s.fock_direct(Da, Db)
        t_ref.append(time.perf_counter() - t0)
        t0 = time.perf_counter()
        J, Ka, _, nq = B.fock_direct(Q, Da + Db, Da)
        t_port.append(time.perf_counter() - t0)
    # The reference returns F = 0 + J - K for D_prev = 0.
    dF = float(np.max(np.abs((J - Ka) - Fa)))
    out = {"system": "(H2O)_16 RHF/6-31G**, 400 bf, core-guess density, full direct build",
           "threads": int(os.environ.get("OMP_NUM_THREADS", os.cpu_count())),
           "reference_s": min(t_ref), "port_s": min(t_port), "port_over_reference": min(t_port) / min(t_ref),
           "surviving_quartets": int(nq), "max_abs_dF": dF, "repeats": repeats}
    print(json.dumps(out), flush=True)


if __name__ == "__main__":
    main()
