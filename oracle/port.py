"""ctypes access to the plain-C restatement of the reference's direct-SCF path (oracle/hf_oracle.c).

Test infrastructure only: the tests, the smoke check and the benchmark's CPU-baseline leg use it as the
checker / the timed CPU arm.  Built by ``build()`` into oracle/liborc.so (git-ignored), the checker, and
into oracle/liborc_rel.so with the reference's release flags (its Makefile:47: -O3 -funroll-loops
-ffp-contract=fast -fno-math-errno -freciprocal-math -fno-trapping-math -fopenmp; without -march=native and
-flto, so that the same recipe builds on x86 and Arm hosts), the timed CPU arm.
"""
from __future__ import annotations

import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
SRC = os.path.join(HERE, "hf_oracle.c")
LIB_PATH = os.path.join(HERE, "liborc.so")
REL_PATH = os.path.join(HERE, "liborc_rel.so")
REL_FLAGS = ["-O3", "-funroll-loops", "-ffp-contract=fast", "-fno-math-errno", "-freciprocal-math",
             "-fno-trapping-math", "-fopenmp"]

_lib = None
_rel = None


def _build_one(path, flags, force):
    if force or not os.path.exists(path) or os.path.getmtime(path) < os.path.getmtime(SRC):
        subprocess.check_call(["gcc"] + flags + ["-fPIC", "-shared", "-std=c11", "-D_GNU_SOURCE", SRC, "-o",
                                                 path + ".tmp", "-lm"])
        os.replace(path + ".tmp", path)
    return path


def build(force: bool = False) -> str:
    _build_one(REL_PATH, REL_FLAGS, force)
    return _build_one(LIB_PATH, ["-O3", "-fopenmp"], force)


class OrcBasis(ctypes.Structure):
    _fields_ = [("nshells", ctypes.c_int), ("nao", ctypes.c_int), ("nprim_total", ctypes.c_int)] + [
        (n, ctypes.POINTER(ctypes.c_int)) for n in ("l", "nprim", "prim_off", "ao_off", "norm_off")
    ] + [(n, ctypes.POINTER(ctypes.c_double)) for n in ("centers", "alpha", "coeff", "norms")] + [
        ("am", ctypes.POINTER(ctypes.c_int))
    ]


def lib(release: bool = False):
    """The checker library, or (release=True) the same code built with the reference's release flags."""
    global _lib, _rel
    if (_rel if release else _lib) is None:
        build()
        L = ctypes.CDLL(REL_PATH if release else LIB_PATH)
        dp, bp, ip = ctypes.POINTER(ctypes.c_double), ctypes.POINTER(OrcBasis), ctypes.POINTER(ctypes.c_int)
        L.orc_boys.argtypes = [ctypes.c_uint, ctypes.c_double, dp]
        L.orc_boys_series.argtypes = [ctypes.c_uint, ctypes.c_double]
        L.orc_boys_series.restype = ctypes.c_double
        L.orc_eri.argtypes = [bp, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long, dp]
        L.orc_schwartz.argtypes = [bp, dp]
        L.orc_survivors.argtypes = [bp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double, ip, ctypes.c_long]
        L.orc_survivors.restype = ctypes.c_long
        L.orc_fock_direct.argtypes = [bp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double, dp, dp, dp]
        L.orc_fock_direct.restype = ctypes.c_long
        L.orc_fock_direct_sample.argtypes = [bp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double,
                                             ctypes.POINTER(ctypes.c_ubyte), dp, dp, dp]
        L.orc_fock_direct_sample.restype = ctypes.c_long
        L.orc_count_survivors.argtypes = [bp, dp, dp, dp, dp, ctypes.c_double, ctypes.c_double]
        L.orc_count_survivors.restype = ctypes.c_long
        L.orc_one_electron.argtypes = [bp, ctypes.c_int, ip, dp, dp, dp, dp]
        L.orc_num_threads.restype = ctypes.c_int
        if release:
            _rel = L
        else:
            _lib = L
    return _rel if release else _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double)) if a is not None else None


class Basis:
    """Keeps the numpy arrays alive behind an OrcBasis view.  ``soa`` uses the keys of the engine's
    structure of arrays: l, nprim, prim_off, ao_off, norm_off, centers (ns,3), alpha, coeff, norms, am (nao,3)."""

    def __init__(self, soa: dict, release: bool = False):
        self.L = lib(release)
        self.arrays = {
            k: np.ascontiguousarray(soa[k], dtype=np.int32 if k in ("l", "nprim", "prim_off", "ao_off", "norm_off", "am") else np.float64)
            for k in ("l", "nprim", "prim_off", "ao_off", "norm_off", "centers", "alpha", "coeff", "norms", "am")
        }
        a = self.arrays
        self.nshells = len(a["l"])
        self.nao = int(sum((l + 1) * (l + 2) // 2 for l in a["l"]))
        self.s = OrcBasis(self.nshells, self.nao, len(a["alpha"]),
                          *[a[k].ctypes.data_as(ctypes.POINTER(ctypes.c_int)) for k in ("l", "nprim", "prim_off", "ao_off", "norm_off")],
                          *[a[k].ctypes.data_as(ctypes.POINTER(ctypes.c_double)) for k in ("centers", "alpha", "coeff", "norms")],
                          a["am"].ctypes.data_as(ctypes.POINTER(ctypes.c_int)))

    def nao_of(self, s):
        l = int(self.arrays["l"][s])
        return (l + 1) * (l + 2) // 2

    def eri(self, a, b, c, d):
        n = [self.nao_of(s) for s in (a, b, c, d)]
        out = np.zeros(int(np.prod(n)))
        self.L.orc_eri(ctypes.byref(self.s), a, b, c, d, _dp(out))
        return out.reshape(n)

    def schwartz(self):
        Q = np.zeros((self.nshells, self.nshells), order="F")
        self.L.orc_schwartz(ctypes.byref(self.s), _dp(Q))
        return Q

    def survivors(self, Q, dDtot, dDa, dDb=None, sthr=1e-10, dthr=1e-10, cap=None):
        args = [np.asfortranarray(x) if x is not None else None for x in (Q, dDtot, dDa, dDb)]
        n = self.L.orc_survivors(ctypes.byref(self.s), *[_dp(x) for x in args], sthr, dthr, None, 0)
        out = np.zeros((n, 4), dtype=np.int32)
        self.L.orc_survivors(ctypes.byref(self.s), *[_dp(x) for x in args], sthr, dthr,
                            out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), n)
        return out

    def fock_direct(self, Q, dDtot, dDa, dDb=None, sthr=1e-10, dthr=1e-10):
        """(J, Ka, Kb or None, survivors) exactly as the reference's direct build forms them."""
        N = self.nao
        J, Ka = np.zeros((N, N), order="F"), np.zeros((N, N), order="F")
        Kb = np.zeros((N, N), order="F") if dDb is not None else None
        args = [np.asfortranarray(x) if x is not None else None for x in (Q, dDtot, dDa, dDb)]
        ns = self.L.orc_fock_direct(ctypes.byref(self.s), *[_dp(x) for x in args], sthr, dthr, _dp(J), _dp(Ka), _dp(Kb))
        return J, Ka, Kb, ns

    def fock_direct_sample(self, Q, dDtot, dDa, bra_mask, dDb=None, sthr=1e-10, dthr=1e-10):
        """The build restricted to the ordered bra pairs (a, b) flagged in bra_mask[a * nshells + b]."""
        N = self.nao
        J, Ka = np.zeros((N, N), order="F"), np.zeros((N, N), order="F")
        Kb = np.zeros((N, N), order="F") if dDb is not None else None
        args = [np.asfortranarray(x) if x is not None else None for x in (Q, dDtot, dDa, dDb)]
        m = np.ascontiguousarray(bra_mask, dtype=np.uint8)
        n = self.L.orc_fock_direct_sample(ctypes.byref(self.s), *[_dp(x) for x in args], sthr, dthr,
                                         m.ctypes.data_as(ctypes.POINTER(ctypes.c_ubyte)), _dp(J), _dp(Ka), _dp(Kb))
        return J, Ka, Kb, n

    def count_survivors(self, Q, dDtot, dDa, dDb=None, sthr=1e-10, dthr=1e-10):
        args = [np.asfortranarray(x) if x is not None else None for x in (Q, dDtot, dDa, dDb)]
        return self.L.orc_count_survivors(ctypes.byref(self.s), *[_dp(x) for x in args], sthr, dthr)

    def one_electron(self, Z, xyz):
        N = self.nao
        S, T, V = (np.zeros((N, N), order="F") for _ in range(3))
        Z = np.ascontiguousarray(Z, dtype=np.int32)
        xyz = np.ascontiguousarray(xyz, dtype=np.float64)
        self.L.orc_one_electron(ctypes.byref(self.s), len(Z), Z.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(xyz), _dp(S), _dp(T), _dp(V))
        return S, T, V


def boys(m_max, T):
    F = np.zeros(m_max + 1)
    lib().orc_boys(m_max, T, _dp(F))
    return F
