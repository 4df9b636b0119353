"""ctypes binding of the hfgpu C ABI (include/hfgpu.h): the Python side of the drop-in boundary.

The library is the in-tree ``libhfgpu.so`` built by ``hfgpu.build``; there is no fallback: if the
library or a GPU is missing, creating an Engine raises.
"""
from __future__ import annotations

import ctypes
import os

import numpy as np

from . import build as _build

HFG_OK = 0
FP64, MIXED = 0, 1
NUM_CLASSES = 21

_lib = None


class _Basis(ctypes.Structure):
    _fields_ = [("nshells", ctypes.c_int), ("nao", ctypes.c_int), ("nprim", ctypes.c_int)] + [
        (n, ctypes.POINTER(ctypes.c_int)) for n in ("l", "nprim_sh", "prim_off", "ao_off", "norm_off")
    ] + [(n, ctypes.POINTER(ctypes.c_double)) for n in ("centers", "alpha", "coeff", "norms")] + [
        ("am", ctypes.POINTER(ctypes.c_int))]


class _Request(ctypes.Structure):
    _fields_ = [("unrestricted", ctypes.c_int), ("precision", ctypes.c_int), ("device_pointers", ctypes.c_int),
                ("schwartz_threshold", ctypes.c_double), ("density_threshold", ctypes.c_double),
                ("fp32_cutoff", ctypes.c_double)] + [
        (n, ctypes.c_void_p) for n in ("dD_tot", "dD_alpha", "dD_beta", "J", "K_alpha", "K_beta")]


class Stats(ctypes.Structure):
    _fields_ = [(n, ctypes.c_ulonglong * NUM_CLASSES) for n in
                ("quartets_fp64", "quartets_fp32", "prim_quartets_fp64", "prim_quartets_fp32")] + [
        (n, ctypes.c_double) for n in ("flops_fp64", "flops_fp32", "ms_total", "ms_lists", "ms_eri_fp64",
                                       "ms_eri_fp32")] + [("kernel_launches", ctypes.c_int)]

    def as_dict(self):
        d = {n: list(getattr(self, n)) for n in ("quartets_fp64", "quartets_fp32", "prim_quartets_fp64",
                                                 "prim_quartets_fp32")}
        d.update({n: getattr(self, n) for n in ("flops_fp64", "flops_fp32", "ms_total", "ms_lists", "ms_eri_fp64",
                                                "ms_eri_fp32", "kernel_launches")})
        return d


def library_path() -> str:
    return _build.LIB_PATH


def lib():
    global _lib
    if _lib is None:
        path = library_path()
        if not os.path.exists(path):
            raise RuntimeError(f"hfgpu library not built: {path} (run __graft_entry__.build())")
        L = ctypes.CDLL(path)
        vp, ip = ctypes.c_void_p, ctypes.c_int
        L.hfg_create.argtypes = [ctypes.POINTER(_Basis), ip, ctypes.POINTER(vp)]
        L.hfg_create_batch.argtypes = [ctypes.POINTER(_Basis), ip, ip, ctypes.POINTER(vp)]
        L.hfg_destroy.argtypes = [vp]
        L.hfg_last_error.argtypes = [vp]
        L.hfg_last_error.restype = ctypes.c_char_p
        L.hfg_schwartz.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        L.hfg_set_schwartz.argtypes = [vp, ctypes.POINTER(ctypes.c_double)]
        L.hfg_fock_direct.argtypes = [vp, ctypes.POINTER(_Request), ctypes.POINTER(Stats)]
        L.hfg_survivors.argtypes = [vp, ctypes.POINTER(ctypes.c_int), ctypes.c_longlong, ctypes.POINTER(ctypes.c_longlong)]
        L.hfg_eri_block.argtypes = [vp, ip, ip, ip, ip, ctypes.POINTER(ctypes.c_double)]
        L.hfg_stream.argtypes = [vp]
        L.hfg_stream.restype = vp
        L.hfg_version.restype = ctypes.c_char_p
        _lib = L
    return _lib


def _dp(a):
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


class HfgError(RuntimeError):
    def __init__(self, code, msg):
        super().__init__(f"hfgpu error {code}: {msg}")
        self.code = code


class _BasisKeep:
    """Keeps the arrays of one molecule's SoA alive behind a _Basis struct."""

    def __init__(self, soa: dict):
        ints = ("l", "nprim", "prim_off", "ao_off", "norm_off", "am")
        self.a = {k: np.ascontiguousarray(soa[k], dtype=np.int32 if k in ints else np.float64) for k in
                  ("l", "nprim", "prim_off", "ao_off", "norm_off", "centers", "alpha", "coeff", "norms", "am")}
        a = self.a
        ip = lambda k: a[k].ctypes.data_as(ctypes.POINTER(ctypes.c_int))
        self.nshells = len(a["l"])
        self.nao = int(sum((int(l) + 1) * (int(l) + 2) // 2 for l in a["l"]))
        self.s = _Basis(self.nshells, self.nao, len(a["alpha"]), ip("l"), ip("nprim"), ip("prim_off"), ip("ao_off"),
                        ip("norm_off"), _dp(a["centers"]), _dp(a["alpha"]), _dp(a["coeff"]), _dp(a["norms"]), ip("am"))


class Engine:
    """One engine over one molecule (soa dict) or a batch (list of soa dicts)."""

    def __init__(self, soa, device: int = 0):
        batch = isinstance(soa, (list, tuple))
        self._keep = [_BasisKeep(s) for s in (soa if batch else [soa])]
        self.nmol = len(self._keep)
        self.naos = [k.nao for k in self._keep]
        self.nshells = [k.nshells for k in self._keep]
        arr = (_Basis * self.nmol)(*[k.s for k in self._keep])
        h = ctypes.c_void_p()
        rc = lib().hfg_create_batch(arr, self.nmol, device, ctypes.byref(h))
        if rc != HFG_OK:
            raise HfgError(rc, lib().hfg_last_error(None).decode())
        self.h = h

    @property
    def nao(self):
        return self.naos[0]

    def close(self):
        if getattr(self, "h", None):
            lib().hfg_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def _check(self, rc):
        if rc != HFG_OK:
            raise HfgError(rc, lib().hfg_last_error(self.h).decode())

    def stream(self) -> int:
        return lib().hfg_stream(self.h)

    def schwartz(self):
        n = sum(ns * ns for ns in self.nshells)
        Q = np.zeros(n)
        self._check(lib().hfg_schwartz(self.h, _dp(Q)))
        if self.nmol == 1:
            ns = self.nshells[0]
            return Q.reshape(ns, ns, order="F")
        return Q

    def set_schwartz(self, Q):
        Q = np.asfortranarray(Q, dtype=np.float64).ravel(order="F")
        self._check(lib().hfg_set_schwartz(self.h, _dp(Q)))

    def fock(self, dD_tot, dD_alpha, dD_beta=None, precision=FP64, sthr=1e-10, dthr=1e-10, fp32_cutoff=1e-6):
        """(J, Ka, Kb or None, stats dict) for host numpy matrices (single molecule: n x n)."""
        uhf = dD_beta is not None
        flat = lambda x: np.asfortranarray(x, dtype=np.float64).ravel(order="F")
        ins = [flat(dD_tot), flat(dD_alpha), flat(dD_beta) if uhf else None]
        size = ins[0].size
        outs = [np.zeros(size) for _ in range(3 if uhf else 2)] + ([] if uhf else [None])
        req = _Request(1 if uhf else 0, precision, 0, sthr, dthr, fp32_cutoff,
                       *[x.ctypes.data if x is not None else None for x in ins],
                       *[x.ctypes.data if x is not None else None for x in outs])
        st = Stats()
        self._check(lib().hfg_fock_direct(self.h, ctypes.byref(req), ctypes.byref(st)))
        if self.nmol == 1:
            n = self.nao
            outs = [o.reshape(n, n, order="F") if o is not None else None for o in outs]
        return outs[0], outs[1], outs[2], st.as_dict()

    def fock_device(self, ptrs: dict, unrestricted=False, precision=FP64, sthr=1e-10, dthr=1e-10, fp32_cutoff=1e-6):
        """Same on device pointers (ints): keys dD_tot, dD_alpha, dD_beta, J, K_alpha, K_beta."""
        g = lambda k: ptrs.get(k) or None
        req = _Request(1 if unrestricted else 0, precision, 1, sthr, dthr, fp32_cutoff, g("dD_tot"), g("dD_alpha"),
                       g("dD_beta"), g("J"), g("K_alpha"), g("K_beta"))
        st = Stats()
        self._check(lib().hfg_fock_direct(self.h, ctypes.byref(req), ctypes.byref(st)))
        return st.as_dict()

    def survivors(self):
        cnt = ctypes.c_longlong()
        self._check(lib().hfg_survivors(self.h, None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, 4), dtype=np.int32)
        self._check(lib().hfg_survivors(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cnt.value,
                                        ctypes.byref(cnt)))
        return out

    def eri_block(self, a, b, c, d):
        ls = self._keep[0].a["l"]
        n = [(int(ls[s]) + 1) * (int(ls[s]) + 2) // 2 for s in (a, b, c, d)]
        out = np.zeros(int(np.prod(n)))
        self._check(lib().hfg_eri_block(self.h, a, b, c, d, _dp(out)))
        return out.reshape(n)
