#!/usr/bin/env python3
"""Benchmark of the GB300 direct-SCF Fock build (one JSON line on stdout, rank 0).

Workload (default): (H2O)_64 on a 4x4x4 lattice, 5.5 bohr spacing, seeded rotations and +-0.2 bohr
jitter (seed 0), RHF/6-31G** with Cartesian d (768 shells, 1600 basis functions); the density is the
core-Hamiltonian guess, so every step is the first (full, non-incremental) direct Fock build of the SCF,
SCHWARTZ_THRESH = DENSITY_THRESH = 1e-10.  A step = one hfg_fock_direct call.

* value      Fock builds/s, mixed FP32/FP64 (quartets whose Q_ab Q_cd max|dD| < 2e-4 in FP32), inputs and
             outputs resident in HBM (device pointers), all ranks' builds / max time over ranks.
* e2e        the same build through the C ABI with host buffers: dD_tot and dD_alpha copied in, J and
             K_alpha copied out, every step.
* fp64_*     the plain all-FP64 GPU build on the same density, and the energy difference of the two
             builds' two-electron energies.
* roofline   the dominant kernel group (the FP64 ERI class kernels), achieved algorithmic FP64 FLOP/s
             (engine work model) over their CUDA-event time, against the FP64 FMA peak this run measures.
* scf        (N=1) full RHF SCFs of the workload, mixed and FP64 (wall time, iterations, |dE|), and the
             mixed-precision nuclear gradient after the mixed SCF; --scf adds the UHF doublet and the FP64
             gradient, --no-scf skips them.
* cpu_baseline / --impl reference   the C restatement of the reference's OpenMP build (oracle/, built
             with the reference's release flags) on this host's cores.  A CPU step is the build over a
             seeded sample of the ordered bra shell pairs of the reference's nShells^4 loop (each sampled
             bra scans its whole ket range): its wall time is measured (ms_per_step) and its Fock builds/s
             is the sampled fraction of the loop over that time; --cpu-full also times one unsampled
             build to check that scaling.

Multi-GPU (torchrun): every rank builds the same workload on its own GPU (independent replicas, no
collective on the data path; weak scaling).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

REPO = os.path.dirname(os.path.abspath(__file__))
for _p in (REPO, os.path.join(REPO, "hartree-fock_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

METRIC = "Fock builds/s & SCF time, (H2O)_64/6-31G**: mixed vs FP64 GPU, |ΔE|≤1e-6 Eh"
# DRAM traffic per mixed build of the ERI class kernels, measured with ncu on the default kernel forms.
ERI_DRAM_BYTES_PER_BUILD = {"h2o64": 12.45e9}
WORKLOADS = {
    "h2o64": dict(lattice=(4, 4, 4), basis="6-31G**", name="(H2O)_64 RHF/6-31G** direct Fock build (1600 bf)"),
    "h2o32": dict(lattice=(4, 4, 2), basis="6-31G**", name="(H2O)_32 RHF/6-31G** direct Fock build (800 bf)"),
    "h2o16": dict(lattice=(4, 2, 2), basis="6-31G**", name="(H2O)_16 RHF/6-31G** direct Fock build (400 bf)"),
}


def parse_args():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["gpu", "reference"], default="gpu")
    ap.add_argument("--workload", choices=sorted(WORKLOADS), default="h2o64")
    ap.add_argument("--fp32-cutoff", type=float, default=2e-4)
    ap.add_argument("--cpu-seconds", type=float, default=15.0, help="target CPU time of one baseline sample")
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--no-tune", action="store_true",
                    help="default kernel form per class, no form-timing trials (the same launches with or without a profiler)")
    ap.add_argument("--scf", action="store_true",
                    help="also time the UHF SCFs and the FP64 gradient (the RHF SCFs and the mixed gradient always run at N=1)")
    ap.add_argument("--no-scf", action="store_true", help="skip the SCF and gradient timings")
    ap.add_argument("--cpu-full", action="store_true",
                    help="--impl reference: also time one full, unsampled CPU build (minutes) against the sampled estimate")
    ap.add_argument("--batch", action="store_true",
                    help="also time batched builds of 256 uneven (H2O)_k/6-31G chains (eager and CUDA-graph replay)")
    return ap.parse_args()


def dist_env():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


class Dist:
    def __init__(self):
        self.world, self.rank, self.local = dist_env()
        self.pg = None
        if self.world > 1:
            import torch
            import torch.distributed as td

            backend = "nccl" if torch.cuda.is_available() else "gloo"
            if backend == "nccl":
                torch.cuda.set_device(self.local)
            td.init_process_group(backend)
            self.td = td
            self.pg = True

    def barrier(self):
        if self.pg:
            import torch

            if torch.cuda.is_available():
                self.td.barrier(device_ids=[self.local])
            else:
                self.td.barrier()

    def max(self, x: float) -> float:
        if not self.pg:
            return x
        import torch

        dev = "cuda" if torch.cuda.is_available() else "cpu"
        t = torch.tensor([x], dtype=torch.float64, device=dev)
        self.td.all_reduce(t, op=self.td.ReduceOp.MAX)
        return float(t.item())

    def close(self):
        if self.pg:
            self.td.destroy_process_group()


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled every 200 ms while active."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.FIELDS}",
                                          "--format=csv,noheader,nounits", "-lms", "200"], stdout=subprocess.PIPE,
                                         stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self):
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9:
                continue
            try:
                sm.append(float(f[1]))
                smax = max(smax, float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def make_workload(name):
    from hfgpu import basis, workloads

    w = WORKLOADS[name]
    Z, xyz = workloads.water_lattice(*w["lattice"], spacing=5.5, seed=0, jitter=0.2)
    soa = basis.pack(w["basis"], Z, xyz)
    return Z, xyz, soa


def cpu_density(soa, Z, xyz):
    """Core-Hamiltonian guess density of the workload on the CPU (the oracle's one-electron integrals and
    numpy's FP64 eigensolver), for the CPU arms, which must not need the GPU."""
    import numpy as np

    from oracle import port

    B = port.Basis(soa)
    S, T, V = B.one_electron(Z, xyz)
    w, U = np.linalg.eigh(S)
    X = (U * np.where(w > 0, 1.0 / np.sqrt(np.maximum(w, 1e-300)), 0.0)) @ U.T
    _, Cp = np.linalg.eigh(X.T @ (T + V) @ X)
    C = X @ Cp
    nocc = sum(Z) // 2
    return C[:, :nocc] @ C[:, :nocc].T


class CpuBuild:
    """The reference's direct Fock build on the host cores: the C restatement of SCF::buildFockMatrixDirect
    (oracle/hf_oracle.c, OpenMP over all host threads) built with the reference's release flags.

    One step runs the build over a seeded random sample of the ordered bra shell pairs (a, b) of the
    reference's nShells^4 loop (SCF.cpp:592-600), scanning each sampled bra's whole ket range with the same
    skip tests, so that a step takes seconds instead of the minutes of a full build and a fraction f of the
    bras costs f of the build, scan included.  Its throughput in Fock builds/s is f over the measured wall
    time of the step; ``full()`` times one unsampled build for the check of that scaling."""

    def __init__(self, soa, Z, xyz, Da, total_quartets=None):
        from oracle import port

        port.build()
        self.B = port.Basis(soa, release=True)
        self.cores = port.lib(True).orc_num_threads()
        self.Q = self.B.schwartz()
        self.dt, self.da = 2.0 * Da, Da
        self.total = int(total_quartets if total_quartets is not None else self.B.count_survivors(self.Q, self.dt, self.da))
        ns = self.B.nshells
        self.npairs = ns * ns  # ordered bra pairs of the nShells^4 loop

    def sample(self, frac, seed):
        import numpy as np

        mask = (np.random.default_rng(seed).random(self.npairs) < frac).astype(np.uint8)
        t0 = time.perf_counter()
        _, _, _, n = self.B.fock_direct_sample(self.Q, self.dt, self.da, mask)
        t = time.perf_counter() - t0
        f = int(mask.sum()) / self.npairs
        return {"seconds": t, "quartets": int(n), "bra_pairs": int(mask.sum()), "fraction": f,
                "quartet_fraction": n / max(self.total, 1), "builds_per_s": f / t if t > 0 else 0.0}

    def calibrate(self, target_s, seed=12345):
        """Sampling fraction whose step takes about target_s seconds."""
        frac = 2e-4
        r = self.sample(frac, seed)
        while r["seconds"] < 0.3 and frac < 0.5:
            frac *= 4
            r = self.sample(frac, seed)
        return min(1.0, frac * target_s / max(r["seconds"], 1e-3))

    def full(self):
        t0 = time.perf_counter()
        _, _, _, n = self.B.fock_direct(self.Q, self.dt, self.da)
        t = time.perf_counter() - t0
        return {"seconds": t, "quartets": int(n), "builds_per_s": 1.0 / t}


def cpu_baseline(workload: str, target_s: float):
    """The GPU arm's cpu_baseline object: the reference arm of this script run in a child process (one
    warm-up and one timed sample of about target_s seconds), so that the OpenMP build runs in a process
    without PyTorch (whose own OpenMP runtime and threads slowed it 3x in the GPU arm's process)."""
    env = {k: v for k, v in os.environ.items()
           if k not in ("RANK", "WORLD_SIZE", "LOCAL_RANK", "LOCAL_WORLD_SIZE", "MASTER_ADDR", "MASTER_PORT")}
    cmd = [sys.executable, os.path.abspath(__file__), "--impl", "reference", "--workload", workload,
           "--steps", "1", "--warmup", "1", "--cpu-seconds", str(target_s / 6.0)]
    r = subprocess.run(cmd, env=env, capture_output=True, text=True, check=True)
    line = json.loads(r.stdout.strip().splitlines()[-1])
    cpu = dict(line["cpu_baseline"])
    cpu["how"] = "child process: bench.py --impl reference --steps 1 --warmup 1 (no PyTorch in the process)"
    return cpu


def reference_arm(args, dist):
    """--impl reference: the reference's direct Fock build on the host cores (CpuBuild), on this arm's
    workload, metric and unit.  Every step is a bounded sample of the build whose wall time is measured;
    ms_per_step is that measured time, and value the median over the steps of sampled fraction / time."""
    if dist.rank != 0:
        return
    Z, xyz, soa = make_workload(args.workload)
    Da = cpu_density(soa, Z, xyz)
    cb = CpuBuild(soa, Z, xyz, Da)
    # Steps sized so that warm-up and timed steps take about --cpu-seconds x 12 in all (3 minutes by default).
    per_step = min(8.0, max(0.5, 12.0 * args.cpu_seconds / max(1, args.steps + args.warmup)))
    frac = cb.calibrate(per_step)
    runs = [cb.sample(frac, seed=i) for i in range(args.warmup + args.steps)][args.warmup:]
    value = statistics.median(r["builds_per_s"] for r in runs)
    ms_step = statistics.median(1000.0 * r["seconds"] for r in runs)
    line = {
        "metric": METRIC, "value": value, "unit": "Fock builds/s", "impl": "reference", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded water lattice)",
        "config": {"workload": WORKLOADS[args.workload]["name"], "precision": "fp64 (reference algorithm)",
                   "step": "the direct build over a seeded random sample of bra shell pairs"},
        "sampling": {"fraction_of_build_per_step": statistics.median(r["fraction"] for r in runs),
                     "quartet_fraction_per_step": statistics.median(r["quartet_fraction"] for r in runs),
                     "quartets_per_step": int(statistics.median(r["quartets"] for r in runs)),
                     "total_quartets": cb.total, "extrapolated_builds_per_s": value,
                     "extrapolated_ms_per_full_build": 1000.0 / value if value else None},
        "cpu_baseline": {"value": value, "unit": "Fock builds/s", "cores": cb.cores, "kind": "port",
                         "sample": (f"{args.steps} steps of {100 * statistics.median(r['fraction'] for r in runs):.3f}% "
                                    f"of the build's surviving quartets each ({ms_step / 1000:.2f} s median, measured)"),
                         "build": "oracle/hf_oracle.c with the reference's release flags (Makefile:47, without "
                                  "-march=native/-flto)"},
        "e2e": {"value": value, "unit": "Fock builds/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "gpu_launches": 0,
    }
    if args.cpu_full:
        line["full_build"] = cb.full()
        line["full_build"]["sampled_estimate_error"] = value / line["full_build"]["builds_per_s"] - 1.0
    print(json.dumps(line), flush=True)


def gpu_arm(args, dist):
    import numpy as np
    import torch

    from hfgpu.engine import FP64, MIXED, Engine, measure_dmma_peak, measure_fma_peak

    dev = dist.local
    torch.cuda.set_device(dev)
    Z, xyz, soa = make_workload(args.workload)
    eng = Engine(soa, device=dev)
    if args.no_tune:
        eng.set_autotune(False)
    Da, _ = eng.core_guess(Z, xyz, 0, 1)
    n = eng.nao
    t64 = lambda a: torch.from_numpy(np.asfortranarray(a).ravel(order="F")).to(f"cuda:{dev}")
    d_dt, d_da = t64(2.0 * Da), t64(Da)
    d_J = torch.zeros(n * n, dtype=torch.float64, device=f"cuda:{dev}")
    d_K = torch.zeros_like(d_J)
    ptrs = dict(dD_tot=d_dt.data_ptr(), dD_alpha=d_da.data_ptr(), J=d_J.data_ptr(), K_alpha=d_K.data_ptr())
    stream = torch.cuda.ExternalStream(eng.stream())
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{dev}")  # > L2 (129 MB)

    def build(prec):
        return eng.fock_device(ptrs, precision=prec, fp32_cutoff=args.fp32_cutoff)

    # Warm-up (also computes the Schwartz matrix and sizes the quartet lists).
    for _ in range(max(args.warmup, 1)):
        st = build(MIXED)
    torch.cuda.synchronize()

    # Timed region: K mixed builds, device resident.
    dist.barrier()
    torch.cuda.synchronize()
    ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    stats = []
    with ClockSampler(dev) as clk:
        ev0.record(stream)
        for _ in range(args.steps):
            with torch.cuda.stream(stream):
                flush.zero_()
            stats.append(build(MIXED))
        ev1.record(stream)
        torch.cuda.synchronize()
    dist.barrier()
    ms = ev0.elapsed_time(ev1)
    ms_max = dist.max(ms)
    value = dist.world * args.steps / (ms_max / 1000.0)
    st = stats[-1]
    J_mixed = d_J.cpu().numpy().reshape(n, n, order="F")
    K_mixed = d_K.cpu().numpy().reshape(n, n, order="F")

    # End to end through the C ABI with pinned host buffers (inputs copied in, J and K copied out per build).
    pinned = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    Dt_h = pinned(np.asfortranarray(2.0 * Da).ravel(order="F"))
    Da_h = pinned(np.asfortranarray(Da).ravel(order="F"))
    out_h = [torch.zeros(n * n, dtype=torch.float64).pin_memory().numpy() for _ in range(2)]
    eng.fock(Dt_h, Da_h, precision=MIXED, fp32_cutoff=args.fp32_cutoff, out=out_h)
    dist.barrier()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        eng.fock(Dt_h, Da_h, precision=MIXED, fp32_cutoff=args.fp32_cutoff, out=out_h)
    e2e_s = dist.max(time.perf_counter() - t0)
    e2e_value = dist.world * args.steps / e2e_s

    # Plain FP64 GPU build on the same density.
    build(FP64)
    torch.cuda.synchronize()
    ev0.record(stream)
    k64 = max(1, min(2, args.steps))
    for _ in range(k64):
        st64 = build(FP64)
    ev1.record(stream)
    torch.cuda.synchronize()
    fp64_value = dist.world * k64 / (dist.max(ev0.elapsed_time(ev1)) / 1000.0)
    J64 = d_J.cpu().numpy().reshape(n, n, order="F")
    K64 = d_K.cpu().numpy().reshape(n, n, order="F")
    # Two-electron energy of the build for the guess density, RHF: E2 = tr(Da (J - K_alpha)).
    e2_mixed = float(np.sum(Da * (J_mixed - K_mixed)))
    e2_fp64 = float(np.sum(Da * (J64 - K64)))

    peak64 = measure_fma_peak(True, dev)
    peak32 = measure_fma_peak(False, dev)
    peak_dmma = measure_dmma_peak(dev)
    # Roofline of the mixed build's ERI class kernels: FP64 and FP32 kernels run concurrently, so the work
    # is weighed as (F64/peak64 + F32/peak32) over their common span, expressed as FP64-equivalent FLOP/s
    # against the FP64 peak.  The FP64 kernels alone are measured in the plain FP64 build.
    t_mix = st["ms_eri_both"] if st["ms_eri_both"] > 0 else st["ms_eri_fp64"] + st["ms_eri_fp32"]
    ach_mix = (st["flops_fp64"] + st["flops_fp32"] * peak64 / peak32) / (t_mix * 1e-3) / 1e12 if t_mix > 0 else 0.0
    ach64 = st64["flops_fp64"] / (st64["ms_eri_fp64"] * 1e-3) / 1e12 if st64["ms_eri_fp64"] > 0 else 0.0
    ach32 = st["flops_fp32"] / (st["ms_eri_fp32"] * 1e-3) / 1e12 if st["ms_eri_fp32"] > 0 else 0.0

    out = None
    if dist.rank == 0:
        cpu = None
        if not args.no_cpu_baseline and dist.world == 1:
            cpu = cpu_baseline(args.workload, args.cpu_seconds)
        out = {
            "metric": METRIC, "value": value, "unit": "Fock builds/s", "n_gpus": dist.world, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": ms_max / args.steps, "higher_is_better": True, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64+f32", "data": "synthetic (seeded water lattice, core-guess density)",
            "config": {"workload": WORKLOADS[args.workload]["name"], "precision": "mixed FP32/FP64",
                       "fp32_cutoff": args.fp32_cutoff, "schwartz_thresh": 1e-10, "density_thresh": 1e-10,
                       "l2": "flushed (256 MB write) before every step", "parallelism": f"replicas x{dist.world}",
                       "kernel_forms": "class defaults (--no-tune)" if args.no_tune else "autotuned on first use"},
            "fp64_builds_per_s": fp64_value,
            "speedup_mixed_vs_fp64": value / fp64_value if fp64_value else None,
            "delta_e2_mixed_vs_fp64": abs(e2_mixed - e2_fp64),
            "max_abs_dF_mixed_vs_fp64": float(max(np.abs(J_mixed - J64).max(), np.abs(K_mixed - K64).max())),
            "quartets": {"fp64": int(sum(st["quartets_fp64"])), "fp32": int(sum(st["quartets_fp32"])),
                         "prim_fp64": int(sum(st["prim_quartets_fp64"])), "prim_fp32": int(sum(st["prim_quartets_fp32"]))},
            "device_ms": {"build": st["ms_total"], "lists": st["ms_lists"], "eri_fp64": st["ms_eri_fp64"],
                          "eri_fp32": st["ms_eri_fp32"], "eri_both_overlapped": st["ms_eri_both"],
                          "fp64_build": st64["ms_total"]},
            "kernel_forms": {"legend": "per quartet class 0-20: 1 thread, 2 warp, 3 group, 0 not launched",
                             "fp64": st["form_fp64"], "fp32": st["form_fp32"], "fp64_only_build": st64["form_fp64"]},
            "roofline": {"bound": "fp64",
                         "kernel": "ERI class kernels of the mixed build (jk_class*_kernel, FP64 and FP32 concurrent)",
                         "achieved": ach_mix, "peak": peak64,
                         "unit": "TFLOP/s (FP64-equivalent: FP32 flops x peak64/peak32, over the kernels' common span)",
                         "frac": ach_mix / peak64 if peak64 else None,
                         "peak_source": "measured FP64 / FP32 FMA loops (hfg_measure_fma_peak) on this GPU",
                         # DRAM bytes (read + write) of the ERI class kernels of one mixed (H2O)_64 build: ncu's
                         # dram__bytes_read.sum + dram__bytes_write.sum over the jk_class kernels of
                         # `bench.py --steps 2 --warmup 3 --no-cpu-baseline --no-scf --no-tune`.
                         "traffic": ERI_DRAM_BYTES_PER_BUILD.get(args.workload),
                         "traffic_unit": "bytes per build (ERI class kernels, ncu)",
                         "traffic_gbs": (ERI_DRAM_BYTES_PER_BUILD[args.workload] / (t_mix * 1e-3) / 1e9
                                         if args.workload in ERI_DRAM_BYTES_PER_BUILD and t_mix > 0 else None),
                         "fp64_kernels_alone": {"achieved": ach64, "peak": peak64, "unit": "TFLOP/s",
                                                "frac": ach64 / peak64 if peak64 else None,
                                                "where": "FP64 class kernels of the plain FP64 build"},
                         "fp32_kernels": {"achieved": ach32, "peak": peak32, "unit": "TFLOP/s",
                                          "frac": ach32 / peak32 if peak32 else None,
                                          "where": "FP32 class kernels over their own span, which overlaps the FP64 span"},
                         "fp64_tensor_dmma_tflops": peak_dmma},
            "e2e": {"value": e2e_value, "unit": "Fock builds/s", "h2d_bytes_per_step": 2 * n * n * 8,
                    "d2h_bytes_per_step": 2 * n * n * 8},
            "gpu_launches": int(sum(s["kernel_launches"] for s in stats)),
            "clocks": clk.summary(),
            "cpu_baseline": cpu,
        }
        if not args.no_scf and dist.world == 1:
            out["scf"] = scf_timings(soa, Z, xyz, dev, args.fp32_cutoff, full=args.scf)
        if args.batch:
            out["batched"] = batch_timings(dev, args.fp32_cutoff, args.steps, args.warmup)
    return out


def scf_timings(soa, Z, xyz, dev, cutoff, full=False):
    """Full SCFs of the workload: RHF in FP64 and mixed precision (the headline speed-up) and the
    mixed-precision nuclear gradient after the mixed SCF; with ``full`` also the FP64 gradient on the same
    densities and the +1 doublet UHF (GUESS_MIX 2) in FP64 and mixed precision."""
    import numpy as np

    from hfgpu.engine import FP64, MIXED, Engine

    def one(prec, charge, mult, grad):
        eng = Engine(soa, device=dev)
        opts = dict(precision=prec, fp32_cutoff=cutoff, energy_tol=1e-8, density_tol=1e-6, diis_tol=1e-6,
                    max_iter=80, unrestricted=int(mult != 1), guess_mix=2 if mult != 1 else 0)
        r, _, _ = eng.scf(Z, xyz, charge, mult, opts)
        out = {"seconds": r["ms_total"] / 1000.0, "fock_seconds": r["ms_fock"] / 1000.0,
               "iterations": r["iterations"], "converged": r["converged"], "e_total": r["e_total"]}
        if mult != 1:
            out["s_squared"] = r["s_squared"]
        if grad:
            # The mixed SCF's gradient: small-bound quartets' derivative integrals in FP32; against the FP64
            # gradient on the same densities when grad == "both".
            t0 = time.perf_counter()
            g, ms2 = eng.gradient(Z, xyz, unrestricted=mult != 1, precision=MIXED, fp32_cutoff=cutoff)
            out["gradient"] = {"precision": "mixed", "seconds": time.perf_counter() - t0, "two_electron_ms": ms2,
                               "max_abs": float(np.abs(g).max()), "sum_abs_translation": float(np.abs(g.sum(0)).max())}
            if grad == "both":
                t0 = time.perf_counter()
                g64, ms64 = eng.gradient(Z, xyz, unrestricted=mult != 1)
                out["gradient"]["fp64_seconds"] = time.perf_counter() - t0
                out["gradient"]["max_abs_vs_fp64_gradient"] = float(np.abs(g - g64).max())
        eng.close()
        return out

    res = {"rhf": {"fp64": one(FP64, 0, 1, False), "mixed": one(MIXED, 0, 1, "both" if full else True)}}
    if full:
        res["uhf_cation_doublet"] = {"fp64": one(FP64, 1, 2, False), "mixed": one(MIXED, 1, 2, True)}
    for k in res:
        res[k]["delta_e"] = abs(res[k]["mixed"]["e_total"] - res[k]["fp64"]["e_total"])
        res[k]["speedup"] = res[k]["fp64"]["seconds"] / res[k]["mixed"]["seconds"]
    return res


def batch_timings(dev, cutoff, steps, warmup):
    """256 independent RHF/6-31G chains (H2O)_k, k ~ U{1..12}: all molecules' builds in one batched
    engine (one list and one launch per quartet class over all molecules), eager and as a replayed CUDA
    graph; aggregate Fock builds/s (molecules x builds / s) and the per-molecule two-electron energy of
    the mixed build against the FP64 build (core-guess densities)."""
    import numpy as np
    import torch

    from hfgpu import basis, workloads
    from hfgpu.engine import FP64, MIXED, Engine

    mols = workloads.uneven_batch(256, 12, seed=0)
    soas = [basis.pack("6-31G", Z, xyz) for Z, xyz in mols]
    dens = []
    for (Z, xyz), soa in zip(mols, soas):
        e1 = Engine(soa, device=dev)
        Da, _ = e1.core_guess(Z, xyz, 0, 1)
        dens.append(Da)
        e1.close()
    eb = Engine(soas, device=dev)
    flat = lambda a: np.asfortranarray(a).ravel(order="F")
    to_dev = lambda a: torch.from_numpy(np.ascontiguousarray(a)).to(f"cuda:{dev}")
    d_dt = to_dev(np.concatenate([flat(2.0 * D) for D in dens]))
    d_da = to_dev(np.concatenate([flat(D) for D in dens]))
    d_J, d_K = torch.zeros_like(d_dt), torch.zeros_like(d_dt)
    ptrs = dict(dD_tot=d_dt.data_ptr(), dD_alpha=d_da.data_ptr(), J=d_J.data_ptr(), K_alpha=d_K.data_ptr())
    stream = torch.cuda.ExternalStream(eb.stream())

    def timed(prec, graph, persistent=False):
        eb.set_persistent(persistent)
        eb.set_graph_mode(graph)
        for _ in range(max(warmup, 3)):
            eb.fock_device(ptrs, precision=prec, fp32_cutoff=cutoff)
        torch.cuda.synchronize()
        ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        ev0.record(stream)
        for _ in range(steps):
            st = eb.fock_device(ptrs, precision=prec, fp32_cutoff=cutoff)
        ev1.record(stream)
        torch.cuda.synchronize()
        ms = ev0.elapsed_time(ev1) / steps
        return ms, st

    def e2_per_molecule():
        J, K = d_J.cpu().numpy(), d_K.cpu().numpy()
        out, off = [], 0
        for D in dens:
            n = D.shape[0]
            Jm = J[off:off + n * n].reshape(n, n, order="F")
            Km = K[off:off + n * n].reshape(n, n, order="F")
            out.append(float(np.sum(D * (Jm - Km))))
            off += n * n
        return np.array(out)

    ms64, st64 = timed(FP64, False)
    e64 = e2_per_molecule()
    ms_mixed, st_mixed = timed(MIXED, False)
    ms_graph, _ = timed(MIXED, True)
    e32 = e2_per_molecule()
    ms_pers, st_pers = timed(MIXED, False, persistent=True)
    e32p = e2_per_molecule()
    ms_pers_graph, _ = timed(MIXED, True, persistent=True)
    eb.set_graph_mode(False)
    eb.set_persistent(False)
    nmol = len(mols)
    return {"molecules": nmol, "basis": "6-31G", "nao_total": int(sum(D.shape[0] for D in dens)),
            "k_range": [1, 12], "seed": 0,
            "fock_builds_per_s": {"fp64": nmol / (ms64 * 1e-3), "mixed": nmol / (ms_mixed * 1e-3),
                                  "mixed_graph": nmol / (ms_graph * 1e-3),
                                  "mixed_persistent": nmol / (ms_pers * 1e-3),
                                  "mixed_persistent_graph": nmol / (ms_pers_graph * 1e-3)},
            "ms_per_batched_build": {"fp64": ms64, "mixed": ms_mixed, "mixed_graph": ms_graph,
                                     "mixed_persistent": ms_pers, "mixed_persistent_graph": ms_pers_graph},
            "kernel_launches_per_build": {"eager": st_mixed["kernel_launches"],
                                          "persistent": st_pers["kernel_launches"], "graph": "1 graph launch"},
            "max_abs_delta_e2_persistent_vs_per_class": float(np.max(np.abs(e32p - e32))),
            "max_abs_delta_e2_per_molecule": float(np.max(np.abs(e32 - e64))),
            "quartets": {"fp64": int(sum(st_mixed["quartets_fp64"])), "fp32": int(sum(st_mixed["quartets_fp32"]))}}


def main():
    args = parse_args()
    dist = Dist()
    try:
        if args.impl == "reference":
            reference_arm(args, dist)
        else:
            out = gpu_arm(args, dist)
            if out is not None:
                print(json.dumps(out), flush=True)
    finally:
        dist.close()


if __name__ == "__main__":
    main()
