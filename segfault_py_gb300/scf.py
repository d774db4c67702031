"""Restricted Hartree-Fock drivers on the GPU (direct SCF).

Same names, arguments and iteration as the reference's src/hf/hf.py:
* ``scf``          hf.py:66-160   plain Roothaan iteration
* ``scf_damping``  hf.py:165-232  density damping 0.1
* ``scf_diis``     hf.py:237-353  cDIIS: error X(FPS - SPF)X, at most 7 vectors
                                  (pop when more than 6 are stored, then append),
                                  DIIS from the third iteration, a singular
                                  Pulay system skips the extrapolation
Convergence is |E_n - E_{n-1}| <= tol, as in the reference.  The difference is
the Fock build: ERIs are never stored; every iteration calls the GPU J/K
builder (FockBuilder.jk), and S, T, V come from the GPU one-electron kernel.
Everything stays on the device in FP64 (eigh, DIIS, energies).
``precision`` ('fp64', 'fp32', 'mixed'), ``cutoff`` and ``fp32_cutoff``
default to the FockBuilder's settings (fp64, 1e-12, 1e-5 for a new one).
"""
from __future__ import annotations

from dataclasses import dataclass, field

import torch

from .fock import DEFAULT_CUTOFF, DEFAULT_FP32_CUTOFF, FockBuilder
from .molecule import Molecule


@dataclass
class SCFResult:
    energy: float                # E_elec + E_nuc
    e_elec: float
    e_nuc: float
    iterations: int
    converged: bool
    D: torch.Tensor = field(repr=False)
    F: torch.Tensor = field(repr=False)
    C: torch.Tensor = field(repr=False)
    eps: torch.Tensor = field(repr=False)
    H: torch.Tensor = field(repr=False)
    S: torch.Tensor = field(repr=False)
    history: list = field(default_factory=list, repr=False)


def preload_torch_linalg():
    """Load torch's CUDA linear-algebra library by absolute path.  torch opens
    it lazily by bare name on the first GPU eigh/solve; under a profiler that
    injects itself into the process that lookup can fail."""
    import ctypes
    import os
    p = os.path.join(os.path.dirname(torch.__file__), "lib", "libtorch_cuda_linalg.so")
    if os.path.exists(p):
        try:
            ctypes.CDLL(p, mode=ctypes.RTLD_GLOBAL)
        except OSError:
            pass


def _setup(mol: Molecule, fb: FockBuilder | None, precision, cutoff, fp32_cutoff, device):
    preload_torch_linalg()
    if fb is None:
        fb = FockBuilder(mol, device=device, cutoff=DEFAULT_CUTOFF if cutoff is None else cutoff,
                         fp32_cutoff=DEFAULT_FP32_CUTOFF if fp32_cutoff is None else fp32_cutoff,
                         precision=precision or "fp64")
    S, T, V = fb.one_electron()
    H = T + V
    vals, vecs = torch.linalg.eigh(S)
    X = vecs @ torch.diag(1.0 / torch.sqrt(vals)) @ vecs.T      # hf.py:278-279
    return fb, S, H, X


def _density(F, X, norb):
    e, Cp = torch.linalg.eigh(X @ F @ X)
    C = X @ Cp
    Co = C[:, :norb]
    return 2.0 * Co @ Co.T, C, e


def _run(mol, mode, tol, maxiter, precision, cutoff, fp32_cutoff, fb, device, damping=0.1, nbuffer=6, dtol=None):
    fb, S, H, X = _setup(mol, fb, precision, cutoff, fp32_cutoff, device)
    norb = mol.nelectron // 2
    F = H.clone()
    etot_old = float("inf")
    counter = 0
    Fs, res, hist = [], [], []
    P_old = torch.zeros_like(H)
    P_prev = None
    converged = False
    while True:
        P_new, C, eps = _density(F, X, norb)
        if mode == "damping":
            P = damping * P_old + (1.0 - damping) * P_new        # hf.py:213-215
            P_old = P_new
        else:
            P = P_new
        J, K = fb.jk(P, precision=precision, cutoff=cutoff, fp32_cutoff=fp32_cutoff)
        F = H + J - 0.5 * K
        etot = float(0.5 * torch.sum(P * (H + F)))
        hist.append(etot + mol.e_nuc)
        dP = float(torch.sqrt(torch.mean((P - P_prev) ** 2))) if (dtol is not None and P_prev is not None) else 0.0
        P_prev = P
        if abs(etot - etot_old) <= tol and (dtol is None or dP <= dtol):
            converged = True
            break
        counter += 1
        etot_old = etot
        if counter > maxiter:
            break
        if mode != "diis" or counter <= 2:
            continue
        if len(Fs) > nbuffer:
            Fs.pop(0)
            res.pop(0)
        res.append(X @ (F @ P @ S - S @ P @ F) @ X)
        Fs.append(F)
        nb = len(Fs) + 1
        B = torch.zeros((nb, nb), dtype=torch.float64, device=F.device)
        B[-1, :] = -1.0
        B[:, -1] = -1.0
        B[-1, -1] = 0.0
        R = torch.stack(res)
        B[:-1, :-1] += torch.einsum("iab,jab->ij", R, R)         # trace(r_i^T r_j)
        rhs = torch.zeros(nb, dtype=torch.float64, device=F.device)
        rhs[-1] = -1.0
        try:
            coef = torch.linalg.solve(B, rhs)
        except RuntimeError:
            continue
        if not bool(torch.isfinite(coef).all()):
            continue
        F = torch.einsum("i,iab->ab", coef[:-1], torch.stack(Fs))
    return SCFResult(energy=etot + mol.e_nuc, e_elec=etot, e_nuc=mol.e_nuc, iterations=counter, converged=converged,
                     D=P, F=F, C=C, eps=eps, H=H, S=S, history=hist)


def scf(mol: Molecule, tol=1e-8, maxiter=30, precision=None, cutoff=None,
        fp32_cutoff=None, fb=None, device="cuda") -> SCFResult:
    """hf.py:66-160 (no convergence acceleration)."""
    return _run(mol, "plain", tol, maxiter, precision, cutoff, fp32_cutoff, fb, device)


def scf_damping(mol: Molecule, tol=1e-8, maxiter=100, precision=None, cutoff=None,
                fp32_cutoff=None, fb=None, device="cuda") -> SCFResult:
    """hf.py:165-232 (one old density mixed in with damping 0.1)."""
    return _run(mol, "damping", tol, maxiter, precision, cutoff, fp32_cutoff, fb, device)


def scf_diis(mol: Molecule, tol=1e-8, maxiter=100, precision=None, cutoff=None,
             fp32_cutoff=None, fb=None, device="cuda", dtol=None) -> SCFResult:
    """hf.py:237-353 (Pulay cDIIS).  ``dtol`` (not in the reference) also
    requires the RMS density change to fall below it, as gradients need."""
    return _run(mol, "diis", tol, maxiter, precision, cutoff, fp32_cutoff, fb, device, dtol=dtol)
