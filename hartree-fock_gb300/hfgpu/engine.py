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
FORM_AUTO, FORM_THREAD, FORM_WARP, FORM_GROUP, FORM_CHUNK = 0, 1, 2, 3, 4

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
                                       "ms_eri_fp32")] + [("kernel_launches", ctypes.c_int),
                                                          ("form_fp64", ctypes.c_int * NUM_CLASSES),
                                                          ("form_fp32", ctypes.c_int * NUM_CLASSES),
                                                          ("ms_tune", ctypes.c_double),
                                                          ("ms_eri_both", ctypes.c_double)]

    def as_dict(self):
        d = {n: list(getattr(self, n)) for n in ("quartets_fp64", "quartets_fp32", "prim_quartets_fp64",
                                                 "prim_quartets_fp32", "form_fp64", "form_fp32")}
        d.update({n: getattr(self, n) for n in ("flops_fp64", "flops_fp32", "ms_total", "ms_lists", "ms_eri_fp64",
                                                "ms_eri_fp32", "kernel_launches", "ms_tune", "ms_eri_both")})
        return d


class ScfOptions(ctypes.Structure):
    _fields_ = [("max_iter", ctypes.c_int), ("energy_tol", ctypes.c_double), ("density_tol", ctypes.c_double),
                ("use_diis", ctypes.c_int), ("diis_size", ctypes.c_int), ("diis_tol", ctypes.c_double),
                ("unrestricted", ctypes.c_int), ("guess_mix", ctypes.c_int), ("damp", ctypes.c_int),
                ("max_damp_iter", ctypes.c_int), ("stop_damp_thresh", ctypes.c_double),
                ("level_shift", ctypes.c_double), ("lshift_gap_tol", ctypes.c_double),
                ("max_lshift_iter", ctypes.c_double), ("stop_lshift_thresh", ctypes.c_double),
                ("schwartz_threshold", ctypes.c_double), ("density_threshold", ctypes.c_double),
                ("precision", ctypes.c_int), ("fp32_cutoff", ctypes.c_double), ("full_rebuild_every", ctypes.c_int),
                ("verbose", ctypes.c_int), ("graph_iterations", ctypes.c_int), ("direct", ctypes.c_int)]


class GradRequest(ctypes.Structure):
    _fields_ = [("natom", ctypes.c_int), ("Z", ctypes.POINTER(ctypes.c_int)), ("xyz", ctypes.POINTER(ctypes.c_double)),
                ("unrestricted", ctypes.c_int), ("D_alpha", ctypes.c_void_p), ("D_beta", ctypes.c_void_p),
                ("W", ctypes.c_void_p), ("schwartz_threshold", ctypes.c_double), ("density_threshold", ctypes.c_double),
                ("precision", ctypes.c_int), ("fp32_cutoff", ctypes.c_double)]


class ScfResult(ctypes.Structure):
    _fields_ = [("e_electronic", ctypes.c_double), ("e_nuclear", ctypes.c_double), ("e_total", ctypes.c_double),
                ("iterations", ctypes.c_int), ("converged", ctypes.c_int), ("delta_e", ctypes.c_double),
                ("delta_d", ctypes.c_double), ("diis_error", ctypes.c_double), ("ms_total", ctypes.c_double),
                ("ms_fock", ctypes.c_double), ("fock_builds", ctypes.c_int), ("s_squared", ctypes.c_double),
                ("graph_replays", ctypes.c_int)]

    def as_dict(self):
        return {n: getattr(self, n) for n, _ in self._fields_}


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
        L.hfg_set_kernel_form.argtypes = [vp, ip, ip, ip]
        L.hfg_set_primitive_threshold.argtypes = [vp, ctypes.c_double]
        L.hfg_set_graph_mode.argtypes = [vp, ip]
        L.hfg_set_persistent.argtypes = [vp, ip]
        L.hfg_set_gradient_form.argtypes = [vp, ip]
        L.hfg_set_autotune.argtypes = [vp, ip]
        L.hfg_set_precision_overlap.argtypes = [vp, ip, ctypes.c_double]
        L.hfg_set_precision_shares.argtypes = [vp, ctypes.c_double, ctypes.c_double]
        L.hfg_kernel_forms.argtypes = [vp, ip, ip, ctypes.POINTER(ctypes.c_int), ctypes.POINTER(ctypes.c_uint)]
        L.hfg_stream.argtypes = [vp]
        L.hfg_stream.restype = vp
        L.hfg_version.restype = ctypes.c_char_p
        dpp = ctypes.POINTER(ctypes.c_double)
        L.hfg_one_electron.argtypes = [ctypes.POINTER(_Basis), ip, ctypes.POINTER(ctypes.c_int), dpp, dpp, dpp, dpp]
        L.hfg_scf_default_options.argtypes = [ctypes.POINTER(ScfOptions), ip]
        L.hfg_scf_default_options.restype = None
        L.hfg_scf_run.argtypes = [vp, ctypes.POINTER(ScfOptions), ip, ctypes.POINTER(ctypes.c_int), dpp, ip, ip,
                                  ctypes.POINTER(ScfResult), dpp, dpp]
        L.hfg_core_guess.argtypes = [vp, ctypes.POINTER(ScfOptions), ip, ctypes.POINTER(ctypes.c_int), dpp, ip, ip,
                                     dpp, dpp]
        L.hfg_measure_fma_peak.argtypes = [ip, ip, dpp]
        L.hfg_measure_dmma_peak.argtypes = [ip, dpp]
        L.hfg_gradient.argtypes = [vp, ctypes.POINTER(GradRequest), dpp, dpp]
        L.hfg_boys_eval.argtypes = [ip, ip, ip, ctypes.c_longlong, dpp, dpp]
        L.hfg_store_integrals.argtypes = [vp, ctypes.c_double, ctypes.POINTER(ctypes.c_size_t)]
        L.hfg_one_electron_gpu.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int), dpp, dpp, dpp, dpp]
        L.hfg_gradient_one_electron_gpu.argtypes = [vp, ip, ctypes.POINTER(ctypes.c_int), dpp, dpp, dpp, dpp]
        L.hfg_gradient_one_electron.argtypes = [ctypes.POINTER(_Basis), ctypes.POINTER(ctypes.c_int), ip,
                                                ctypes.POINTER(ctypes.c_int), dpp, dpp, dpp, dpp]
        L.hfg_fock_conventional.argtypes = [vp, ctypes.POINTER(_Request), ctypes.POINTER(Stats)]
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

    def fock(self, dD_tot, dD_alpha, dD_beta=None, precision=FP64, sthr=1e-10, dthr=1e-10, fp32_cutoff=2e-4,
             out=None):
        """(J, Ka, Kb or None, stats dict) for host numpy matrices (single molecule: n x n).  `out`: optional
        caller-owned flat float64 host buffers [J, Ka(, Kb)] (e.g. pinned memory) that receive the result."""
        uhf = dD_beta is not None
        flat = lambda x: np.asfortranarray(x, dtype=np.float64).ravel(order="F")
        ins = [flat(dD_tot), flat(dD_alpha), flat(dD_beta) if uhf else None]
        size = ins[0].size
        if out is not None:
            outs = list(out) + ([] if uhf else [None])
            if any(o.dtype != np.float64 or o.size != size or not o.flags.c_contiguous for o in outs if o is not None):
                raise ValueError("fock: out buffers must be contiguous float64 arrays of the matrix size")
        else:
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

    def one_electron(self, Z, xyz):
        """S, T, V of this engine's molecule computed on the GPU (FP64)."""
        n = self.nao
        S, T, V = (np.zeros((n, n), order="F") for _ in range(3))
        Zc = np.ascontiguousarray(Z, dtype=np.int32)
        X = np.ascontiguousarray(xyz, dtype=np.float64)
        self._check(lib().hfg_one_electron_gpu(self.h, len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(X),
                                               _dp(S), _dp(T), _dp(V)))
        return S, T, V

    def gradient_one_electron(self, Z, xyz, D, W):
        """sum D d(T+V)/dX - W dS/dX on the GPU (natom x 3); D total density, W energy-weighted density."""
        Zc = np.ascontiguousarray(Z, dtype=np.int32)
        X = np.ascontiguousarray(xyz, dtype=np.float64)
        g = np.zeros((len(Zc), 3))
        Df, Wf = (np.asfortranarray(a, dtype=np.float64) for a in (D, W))
        self._check(lib().hfg_gradient_one_electron_gpu(self.h, len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                                        _dp(X), _dp(Df), _dp(Wf), _dp(g)))
        return g

    def store_integrals(self, sthr=1e-10) -> int:
        """Evaluate and keep every Schwartz-surviving integral (the DIRECT FALSE path); returns the bytes."""
        b = ctypes.c_size_t()
        self._check(lib().hfg_store_integrals(self.h, sthr, ctypes.byref(b)))
        return b.value

    def fock_conventional(self, D_tot, D_alpha, D_beta=None, sthr=1e-10):
        """(J, Ka, Kb or None, stats) of the FULL densities from the stored integrals (host matrices)."""
        uhf = D_beta is not None
        flat = lambda x: np.asfortranarray(x, dtype=np.float64).ravel(order="F")
        ins = [flat(D_tot), flat(D_alpha), flat(D_beta) if uhf else None]
        outs = [np.zeros(ins[0].size) for _ in range(3 if uhf else 2)] + ([] if uhf else [None])
        req = _Request(1 if uhf else 0, FP64, 0, sthr, 0.0, 0.0, *[x.ctypes.data if x is not None else None for x in ins],
                       *[x.ctypes.data if x is not None else None for x in outs])
        st = Stats()
        self._check(lib().hfg_fock_conventional(self.h, ctypes.byref(req), ctypes.byref(st)))
        n = self.nao
        outs = [o.reshape(n, n, order="F") if o is not None else None for o in outs]
        return outs[0], outs[1], outs[2], st.as_dict()

    def fock_device(self, ptrs: dict, unrestricted=False, precision=FP64, sthr=1e-10, dthr=1e-10, fp32_cutoff=2e-4):
        """Same on device pointers (ints): keys dD_tot, dD_alpha, dD_beta, J, K_alpha, K_beta."""
        g = lambda k: ptrs.get(k) or None
        req = _Request(1 if unrestricted else 0, precision, 1, sthr, dthr, fp32_cutoff, g("dD_tot"), g("dD_alpha"),
                       g("dD_beta"), g("J"), g("K_alpha"), g("K_beta"))
        st = Stats()
        self._check(lib().hfg_fock_direct(self.h, ctypes.byref(req), ctypes.byref(st)))
        return st.as_dict()

    def set_precision_overlap(self, on: bool, share: float = 1.0):
        """Run a mixed build's FP32 class kernels concurrently with the FP64 ones (grids at `share` of the
        resident blocks per SM)."""
        self._check(lib().hfg_set_precision_overlap(self.h, 1 if on else 0, float(share)))

    def set_precision_shares(self, share_fp64: float, share_fp32: float):
        """Grid limits of the overlapped FP64 and FP32 class kernels, separately."""
        self._check(lib().hfg_set_precision_shares(self.h, float(share_fp64), float(share_fp32)))

    def set_graph_mode(self, on: bool):
        """Replay device-pointer Fock builds as CUDA graphs (captured on first use per request key)."""
        self._check(lib().hfg_set_graph_mode(self.h, 1 if on else 0))

    def set_persistent(self, on: bool):
        """Run the small classes of both precisions as one persistent work-queue launch."""
        self._check(lib().hfg_set_persistent(self.h, 1 if on else 0))

    def set_autotune(self, on: bool):
        """Time the kernel forms of a class on its first large build (default) or run the default forms only."""
        self._check(lib().hfg_set_autotune(self.h, 1 if on else 0))

    def set_gradient_form(self, group_only: bool):
        """Gradient kernels: the lane-group form for every class (True) or the thread form where compiled."""
        self._check(lib().hfg_set_gradient_form(self.h, 1 if group_only else 0))

    def set_primitive_threshold(self, threshold: float):
        """Primitive-pair screening of the Fock build (0 keeps every primitive pair; default 1e-15)."""
        self._check(lib().hfg_set_primitive_threshold(self.h, float(threshold)))

    def set_kernel_form(self, form, qclass=-1, fp32=False):
        """Force a kernel form (FORM_THREAD / FORM_WARP / FORM_GROUP / FORM_CHUNK) or return to FORM_AUTO."""
        self._check(lib().hfg_set_kernel_form(self.h, qclass, 1 if fp32 else 0, form))

    def kernel_forms(self, fp32=False, unrestricted=False):
        """(forms in use per class, 0 = not tuned yet; bit masks of the compiled forms)."""
        forms = (ctypes.c_int * NUM_CLASSES)()
        avail = (ctypes.c_uint * NUM_CLASSES)()
        self._check(lib().hfg_kernel_forms(self.h, 1 if fp32 else 0, 1 if unrestricted else 0, forms, avail))
        return list(forms), list(avail)

    def survivors(self):
        cnt = ctypes.c_longlong()
        self._check(lib().hfg_survivors(self.h, None, 0, ctypes.byref(cnt)))
        out = np.zeros((cnt.value, 4), dtype=np.int32)
        self._check(lib().hfg_survivors(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), cnt.value,
                                        ctypes.byref(cnt)))
        return out

    def _opts(self, opts: dict, multiplicity: int) -> ScfOptions:
        o = ScfOptions()
        lib().hfg_scf_default_options(ctypes.byref(o), multiplicity)
        for k, v in (opts or {}).items():
            setattr(o, k, v)
        return o

    def scf(self, Z, xyz, charge=0, multiplicity=1, opts: dict | None = None):
        """Full direct SCF on this engine's molecule; returns (result dict, Da, Db)."""
        o = self._opts(opts, multiplicity)
        Zc = np.ascontiguousarray(Z, dtype=np.int32)
        X = np.ascontiguousarray(xyz, dtype=np.float64)
        n = self.nao
        Da, Db = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        r = ScfResult()
        self._check(lib().hfg_scf_run(self.h, ctypes.byref(o), len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                      _dp(X), charge, multiplicity, ctypes.byref(r), _dp(Da), _dp(Db)))
        return r.as_dict(), Da, Db

    def core_guess(self, Z, xyz, charge=0, multiplicity=1, opts: dict | None = None):
        o = self._opts(opts, multiplicity)
        Zc = np.ascontiguousarray(Z, dtype=np.int32)
        X = np.ascontiguousarray(xyz, dtype=np.float64)
        n = self.nao
        Da, Db = np.zeros((n, n), order="F"), np.zeros((n, n), order="F")
        self._check(lib().hfg_core_guess(self.h, ctypes.byref(o), len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)),
                                         _dp(X), charge, multiplicity, _dp(Da), _dp(Db)))
        return Da, Db

    def gradient(self, Z, xyz, Da=None, Db=None, W=None, unrestricted=False, sthr=1e-10, dthr=1e-10,
                 precision=FP64, fp32_cutoff=2e-4):
        """Nuclear gradient (natom x 3, Eh/bohr) and the two-electron device time in ms.  With Da None the
        densities of this engine's last scf() are used (the backward half of scf()).  precision MIXED runs
        the small-bound quartets' derivative integrals in FP32."""
        Zc = np.ascontiguousarray(Z, dtype=np.int32)
        X = np.ascontiguousarray(xyz, dtype=np.float64)
        arrs = [np.asfortranarray(m, dtype=np.float64) if m is not None else None for m in (Da, Db, W)]
        ptr = lambda m: m.ctypes.data if m is not None else None
        req = GradRequest(len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(X), 1 if unrestricted else 0,
                          *[ptr(m) for m in arrs], sthr, dthr, precision, fp32_cutoff)
        g = np.zeros((len(Zc), 3))
        ms = ctypes.c_double()
        self._check(lib().hfg_gradient(self.h, ctypes.byref(req), _dp(g), ctypes.byref(ms)))
        return g, ms.value

    def eri_block(self, a, b, c, d):
        ls = self._keep[0].a["l"]
        n = [(int(ls[s]) + 1) * (int(ls[s]) + 2) // 2 for s in (a, b, c, d)]
        out = np.zeros(int(np.prod(n)))
        self._check(lib().hfg_eri_block(self.h, a, b, c, d, _dp(out)))
        return out.reshape(n)


def one_electron(soa: dict, Z, xyz):
    """(S, T, V) host FP64 through hfg_one_electron."""
    k = _BasisKeep(soa)
    n = k.nao
    S, T, V = (np.zeros((n, n), order="F") for _ in range(3))
    Zc = np.ascontiguousarray(Z, dtype=np.int32)
    X = np.ascontiguousarray(xyz, dtype=np.float64)
    rc = lib().hfg_one_electron(ctypes.byref(k.s), len(Zc), Zc.ctypes.data_as(ctypes.POINTER(ctypes.c_int)), _dp(X),
                                _dp(S), _dp(T), _dp(V))
    if rc != HFG_OK:
        raise HfgError(rc, "hfg_one_electron failed")
    return S, T, V


def measure_fma_peak(fp64: bool, device: int = 0) -> float:
    """TFLOP/s of a register-only FMA loop on this GPU (FP64 or FP32 CUDA cores)."""
    t = ctypes.c_double()
    rc = lib().hfg_measure_fma_peak(device, 1 if fp64 else 0, ctypes.byref(t))
    if rc != HFG_OK:
        raise HfgError(rc, "hfg_measure_fma_peak failed")
    return t.value


def boys_eval(m_max: int, T, fp32: bool = False, device: int = 0) -> np.ndarray:
    """F_0(T) .. F_m_max(T) from the device Boys function of the ERI kernels; returns (len(T), m_max + 1)."""
    T = np.ascontiguousarray(T, dtype=np.float64).ravel()
    F = np.zeros((T.size, m_max + 1))
    rc = lib().hfg_boys_eval(device, m_max, 1 if fp32 else 0, T.size, _dp(T), _dp(F))
    if rc != HFG_OK:
        raise HfgError(rc, "hfg_boys_eval failed")
    return F


def measure_dmma_peak(device: int = 0) -> float:
    """TFLOP/s of a register-only FP64 tensor-core (DMMA m8n8k4) loop on this GPU."""
    t = ctypes.c_double()
    rc = lib().hfg_measure_dmma_peak(device, ctypes.byref(t))
    if rc != HFG_OK:
        raise HfgError(rc, "hfg_measure_dmma_peak failed")
    return t.value


def run_input(text: str, precision: int = FP64, fp32_cutoff: float = 2e-4, full_rebuild_every: int = 0,
              basis_dir: str | None = None, device: int = 0, graphs: bool = False, input_frame: bool = False):
    """Runs a reference-format input end to end: parse, pack the basis, GPU direct SCF (graphs: replay
    the Fock builds of the SCF iterations as CUDA graphs).

    SYMMETRY TRUE (the reference's default) makes the reference move the molecule to its centre of mass
    and rotate it into its point-group frame (src/Molecule.cpp:19-27) before anything is computed.  hfgpu
    does not detect point groups, so such an input raises ValueError unless ``input_frame`` is True, which
    runs the molecule as given: the energy is the same (it is invariant under rigid motions), densities
    and gradients are in the input frame."""
    from . import basis as _basis, inputs as _inputs

    job = _inputs.parse(text)
    _inputs.check_supported(job, input_frame)
    soa = _basis.pack(job.basis, job.Z, job.xyz, basis_dir)
    eng = Engine(soa, device=device)
    if graphs:
        eng.set_graph_mode(True)
    opts = _inputs.scf_options(job, precision, fp32_cutoff, full_rebuild_every)
    res, Da, Db = eng.scf(job.Z, job.xyz, job.charge, job.multiplicity, opts)
    return res, Da, Db, eng
