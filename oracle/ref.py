"""ctypes access to the reference program compiled as the CPU oracle (oracle/_ref/libhfref.so).

Test infrastructure only.  The library is built from the reference's own sources by
oracle/Makefile.ref wherever those sources are present; elsewhere ``available()`` is False and the
tests that need it are skipped (committed golden fixtures under tests/golden stand in for it).
"""
from __future__ import annotations

import ctypes
import os
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
LIB_PATH = os.path.join(REF_DIR, "libhfref.so")

_lib = None


def available() -> bool:
    return os.path.exists(LIB_PATH)


def lib():
    global _lib
    if _lib is None:
        L = ctypes.CDLL(LIB_PATH)
        vp, dp, ip, lp = ctypes.c_void_p, ctypes.POINTER(ctypes.c_double), ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_long)
        L.ref_open.restype = vp
        L.ref_open.argtypes = [ctypes.c_char_p, ctypes.c_char_p, ctypes.c_char_p]
        L.ref_close.argtypes = [vp]
        L.ref_last_error.restype = ctypes.c_char_p
        L.ref_info.argtypes = [vp, lp, dp]
        L.ref_geometry.argtypes = [vp, ip, dp]
        L.ref_basis_soa.argtypes = [vp, ip, ip, ip, ip, ip, dp, dp, dp, dp, ip]
        L.ref_boys.argtypes = [ctypes.c_uint, ctypes.c_double, dp]
        L.ref_boys_analytical.argtypes = [ctypes.c_uint, ctypes.c_double]
        L.ref_boys_analytical.restype = ctypes.c_double
        L.ref_eri.argtypes = [vp, ctypes.c_long, ctypes.c_long, ctypes.c_long, ctypes.c_long, dp]
        L.ref_schwartz.argtypes = [vp, dp]
        L.ref_one_electron.argtypes = [vp, dp, dp, dp]
        L.ref_guess.argtypes = [vp, dp, dp]
        L.ref_fock_direct.argtypes = [vp, dp, dp, dp, dp, dp, dp, dp, dp]
        L.ref_scf_run.argtypes = [vp, dp, dp, dp, dp, dp]
        _lib = L
    return _lib


def _p(a, t=ctypes.c_double):
    return a.ctypes.data_as(ctypes.POINTER(t))


def boys(m_max: int, T: float) -> np.ndarray:
    F = np.zeros(m_max + 1)
    lib().ref_boys(m_max, T, _p(F))
    return F


def boys_analytical(m: int, T: float) -> float:
    return lib().ref_boys_analytical(m, T)


class RefSession:
    """One parsed input: reference SCF object after initialize() and the core guess."""

    def __init__(self, input_text: str):
        self._dir = tempfile.mkdtemp(prefix="hfref_")
        self.input_path = os.path.join(self._dir, "job.in")
        with open(self.input_path, "w") as f:
            f.write(input_text)
        out = os.path.join(self._dir, "job.out")
        self.h = lib().ref_open(self.input_path.encode(), REF_DIR.encode(), out.encode())
        if not self.h:
            raise RuntimeError(lib().ref_last_error().decode())
        sizes = np.zeros(8, dtype=np.int64)
        enuc = np.zeros(1)
        lib().ref_info(self.h, _p(sizes, ctypes.c_long), _p(enuc))
        (self.nshells, self.nao, self.nprim, self.nnorm, unr, self.nocc_a, self.nocc_b, self.natom) = [int(v) for v in sizes]
        self.unrestricted = bool(unr)
        self.nuclear_repulsion = float(enuc[0])

    def close(self):
        if self.h:
            lib().ref_close(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def geometry(self):
        Z = np.zeros(self.natom, dtype=np.int32)
        xyz = np.zeros((self.natom, 3))
        lib().ref_geometry(self.h, _p(Z, ctypes.c_int), _p(xyz))
        return Z, xyz

    def basis_soa(self) -> dict:
        ns = self.nshells
        d = dict(
            l=np.zeros(ns, np.int32), nprim=np.zeros(ns, np.int32), prim_off=np.zeros(ns, np.int32),
            ao_off=np.zeros(ns, np.int32), norm_off=np.zeros(ns, np.int32), centers=np.zeros((ns, 3)),
            alpha=np.zeros(self.nprim), coeff=np.zeros(self.nprim), norms=np.zeros(self.nnorm),
            am=np.zeros((self.nao, 3), np.int32),
        )
        I = ctypes.c_int
        lib().ref_basis_soa(self.h, _p(d["l"], I), _p(d["nprim"], I), _p(d["prim_off"], I), _p(d["ao_off"], I),
                            _p(d["norm_off"], I), _p(d["centers"]), _p(d["alpha"]), _p(d["coeff"]),
                            _p(d["norms"]), _p(d["am"], I))
        return d

    def nao_of(self, s):
        l = self.basis_soa()["l"][s]
        return (l + 1) * (l + 2) // 2

    def eri(self, a, b, c, d) -> np.ndarray:
        soa = self.basis_soa() if not hasattr(self, "_soa") else self._soa
        self._soa = soa
        n = [(soa["l"][s] + 1) * (soa["l"][s] + 2) // 2 for s in (a, b, c, d)]
        out = np.zeros(int(np.prod(n)))
        lib().ref_eri(self.h, a, b, c, d, _p(out))
        return out.reshape(n)

    def schwartz(self) -> np.ndarray:
        Q = np.zeros((self.nshells, self.nshells), order="F")
        lib().ref_schwartz(self.h, _p(Q))
        return Q

    def one_electron(self):
        n = self.nao
        S, T, V = (np.zeros((n, n), order="F") for _ in range(3))
        lib().ref_one_electron(self.h, _p(S), _p(T), _p(V))
        return S, T, V

    def guess(self):
        n = self.nao
        Da, Db = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        lib().ref_guess(self.h, _p(Da), _p(Db))
        return Da, Db

    def fock_direct(self, Da, Db, Da_prev=None, Db_prev=None, Fa_prev=None, Fb_prev=None):
        """F = F_prev + J[dD_tot] - K[dD_spin] through SCF::buildFockMatrixDirect."""
        n = self.nao
        z = np.zeros((n, n), order="F")
        args = [np.asfortranarray(x if x is not None else z, dtype=np.float64)
                for x in (Da, Db, Da_prev, Db_prev, Fa_prev, Fb_prev)]
        Fa, Fb = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        rc = lib().ref_fock_direct(self.h, *[_p(a) for a in args], _p(Fa), _p(Fb))
        if rc != 0:
            raise RuntimeError(lib().ref_last_error().decode())
        return Fa, Fb

    def scf_run(self):
        n = self.nao
        out = np.zeros(3)
        mats = [np.zeros((n, n), order="F") for _ in range(4)]
        rc = lib().ref_scf_run(self.h, _p(out), *[_p(m) for m in mats])
        if rc != 0:
            raise RuntimeError(lib().ref_last_error().decode())
        return dict(e_elec=out[0], e_nuc=out[1], iterations=int(out[2]), Da=mats[0], Db=mats[1], Fa=mats[2], Fb=mats[3])
