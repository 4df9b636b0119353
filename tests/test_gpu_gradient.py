"""Analytic nuclear gradient (adjoint GPU kernel + host one-electron terms) against central finite
differences (+-1e-4 bohr) of the reference program's SCF energy, tolerance 1e-5 Eh/bohr; translational
invariance; and the forward/backward pair through a torch.autograd.Function used only here."""
import os

import numpy as np
import pytest

from conftest import GOLDEN

pytestmark = pytest.mark.gpu

FD_NAMES = sorted(f[:-4] for f in os.listdir(GOLDEN) if f.startswith("fd_") and f.endswith(".npz"))
TIGHT = dict(energy_tol=1e-11, density_tol=1e-9, diis_tol=1e-9, max_iter=300, schwartz_threshold=1e-14,
             density_threshold=1e-14)


def load_fd(name):
    return dict(np.load(os.path.join(GOLDEN, name + ".npz")))


def scf_and_gradient(g, precision=0):
    from hfgpu import basis
    from hfgpu.engine import Engine

    Z, xyz = g["Z"], g["xyz"]
    mult = int(g["multiplicity"])
    opts = dict(TIGHT, precision=precision, unrestricted=int(mult != 1),
                guess_mix=2 if "GUESS_MIX" in str(g["extra"]) else 0)
    e = Engine(basis.pack(str(g["basis"]), Z, xyz))
    res, Da, Db = e.scf(Z, xyz, int(g["charge"]), mult, opts)
    grad, ms = e.gradient(Z, xyz, sthr=1e-14, dthr=1e-14)
    return res, grad


@pytest.mark.parametrize("name", FD_NAMES)
def test_gradient_matches_reference_finite_differences(name):
    g = load_fd(name)
    res, grad = scf_and_gradient(g)
    assert res["converged"] == 1
    assert abs(res["e_total"] - float(g["energy"])) <= 1e-8
    assert np.max(np.abs(grad - g["grad_fd"])) <= 1e-5, np.abs(grad - g["grad_fd"]).max()
    # Translational invariance of the analytic gradient.
    assert np.max(np.abs(grad.sum(axis=0))) <= 1e-8


def test_gradient_through_autograd_function():
    torch = pytest.importorskip("torch")
    from hfgpu import basis
    from hfgpu.engine import Engine

    g = load_fd("fd_h2o_631g")
    Z = g["Z"]

    class HFEnergy(torch.autograd.Function):
        """Forward: direct SCF energy (hfg_scf_run).  Backward: hfg_gradient of the same engine."""

        @staticmethod
        def forward(ctx, xyz):
            x = xyz.detach().cpu().numpy().astype(np.float64)
            e = Engine(basis.pack(str(g["basis"]), Z, x))
            res, _, _ = e.scf(Z, x, 0, 1, TIGHT)
            grad, _ = e.gradient(Z, x, sthr=1e-14, dthr=1e-14)
            ctx.save_for_backward(torch.from_numpy(grad))
            return torch.tensor(res["e_total"], dtype=torch.float64)

        @staticmethod
        def backward(ctx, gout):
            (grad,) = ctx.saved_tensors
            return gout * grad

    xyz = torch.tensor(g["xyz"], dtype=torch.float64, requires_grad=True)
    E = HFEnergy.apply(xyz)
    E.backward()
    assert abs(float(E.detach()) - float(g["energy"])) <= 1e-8
    assert np.max(np.abs(xyz.grad.numpy() - g["grad_fd"])) <= 1e-5


def test_gradient_mixed_precision_close_to_fp64():
    g = load_fd("fd_w2_631gss")
    _, g64 = scf_and_gradient(g, precision=0)
    _, g32 = scf_and_gradient(g, precision=1)
    assert np.max(np.abs(g32 - g64)) <= 1e-5


@pytest.mark.parametrize("name", ["fd_w2_631gss", "fd_h2o_cation_uhf_631g"])
def test_gradient_fp32_split_matches_fp64_and_fd(name):
    """Mixed-precision two-electron gradient (small-bound quartets' derivative integrals in FP32, FP64
    accumulation) on the same converged densities as the FP64 one: within 1e-6 Eh/bohr of it and within
    the finite-difference tolerance of the reference energy."""
    from hfgpu import basis
    from hfgpu.engine import Engine

    g = load_fd(name)
    Z, xyz = g["Z"], g["xyz"]
    mult = int(g["multiplicity"])
    opts = dict(TIGHT, unrestricted=int(mult != 1), guess_mix=2 if "GUESS_MIX" in str(g["extra"]) else 0)
    e = Engine(basis.pack(str(g["basis"]), Z, xyz))
    res, _, _ = e.scf(Z, xyz, int(g["charge"]), mult, opts)
    assert res["converged"] == 1
    g64, _ = e.gradient(Z, xyz, unrestricted=mult != 1, sthr=1e-14, dthr=1e-14)
    g32, _ = e.gradient(Z, xyz, unrestricted=mult != 1, sthr=1e-14, dthr=1e-14, precision=1, fp32_cutoff=1e-4)
    assert np.max(np.abs(g32 - g64)) <= 1e-6
    assert np.max(np.abs(g32 - g["grad_fd"])) <= 1e-5
    assert np.max(np.abs(g32.sum(axis=0))) <= 1e-8


@pytest.mark.parametrize("name", ["fd_w2_631gss", "fd_h2o_cation_uhf_631g"])
def test_gradient_thread_form_matches_group_form(name):
    """The thread-per-quartet gradient kernel (small classes) and the lane-group kernel (every class) give
    the same two-electron gradient on the same densities: FP64 within 1e-11 Eh/bohr, mixed precision
    within 1e-7 (FP32 derivative integrals, summed in a different order); the thread form also within
    the finite-difference tolerance of the reference energy."""
    from hfgpu import basis
    from hfgpu.engine import Engine

    g = load_fd(name)
    Z, xyz = g["Z"], g["xyz"]
    mult = int(g["multiplicity"])
    opts = dict(TIGHT, unrestricted=int(mult != 1), guess_mix=2 if "GUESS_MIX" in str(g["extra"]) else 0)
    e = Engine(basis.pack(str(g["basis"]), Z, xyz))
    res, _, _ = e.scf(Z, xyz, int(g["charge"]), mult, opts)
    assert res["converged"] == 1
    kw = dict(unrestricted=mult != 1, sthr=1e-14, dthr=1e-14)
    out = {}
    for group_only in (False, True):
        e.set_gradient_form(group_only)
        out[group_only] = (e.gradient(Z, xyz, **kw)[0], e.gradient(Z, xyz, precision=1, fp32_cutoff=1e-4, **kw)[0])
    e.set_gradient_form(False)
    assert np.max(np.abs(out[False][0] - out[True][0])) <= 1e-11
    assert np.max(np.abs(out[False][1] - out[True][1])) <= 1e-7
    assert np.max(np.abs(out[False][0] - g["grad_fd"])) <= 1e-5
