"""Analytic RHF nuclear gradients and the differentiable RHF energy.

The reference computes energies only.  Here

    dE/dR_A = sum_pq D_pq dH_pq/dR_A - sum_pq W_pq dS_pq/dR_A
              + sum_pqrs G_pqrs d(pq|rs)/dR_A + dE_nuc/dR_A,
    G_pqrs = 1/2 D_pq D_rs - 1/8 (D_pr D_qs + D_ps D_qr),
    W = 2 sum_occ e_i C_pi C_qi = (D F D)/2 at the converged density,

with the derivative integrals contracted on the GPU (sf_grad_one_electron,
sf_grad_jk) and the nuclear term on the host.  ``RHFEnergy`` wraps the SCF
energy as a torch.autograd.Function whose backward returns these forces.
Coordinates are in bohr, gradients in Eh/bohr.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .fock import FockBuilder, _ptr, _stream_ptr
from .molecule import BOHR, Molecule
from .scf import SCFResult, scf_diis


def nuclear_repulsion_gradient(mol: Molecule) -> np.ndarray:
    """d/dR_A of sum_{A<B} Z_A Z_B / |R_A - R_B| (molecule.py:75-80)."""
    R = np.asarray(mol.xyz__, dtype=np.float64)
    Z = mol.numbers.astype(np.float64)
    d = R[:, None, :] - R[None, :, :]                  # R_A - R_B
    r = np.linalg.norm(d, axis=2)
    np.fill_diagonal(r, np.inf)
    return -np.einsum("ab,abk->ak", np.outer(Z, Z) / r ** 3, d)


def energy_weighted_density(F: torch.Tensor, X: torch.Tensor, norb: int):
    """D = 2 C_occ C_occ^T and W = 2 C_occ diag(e_occ) C_occ^T from F."""
    e, Cp = torch.linalg.eigh(X @ F @ X)
    Cm = X @ Cp
    Co = Cm[:, :norb]
    D = 2.0 * Co @ Co.T
    W = 2.0 * (Co * e[:norb]) @ Co.T
    return D, W


def rhf_gradient(mol: Molecule, res: SCFResult, fb: FockBuilder, precision: str | None = None,
                 cutoff: float | None = None, fp32_cutoff: float | None = None) -> torch.Tensor:
    """(natom, 3) gradient in Eh/bohr at the converged SCF ``res``."""
    L = _lib.lib()
    dev = fb.device
    # at the converged SCF: D = 2 C_occ C_occ^T and W = 2 C_occ (C_occ^T F C_occ)
    # C_occ^T = D F D / 2, orbital-invariant (no diagonalisation needed)
    D = res.D.contiguous()
    W = (0.5 * (D @ res.F @ D)).contiguous()
    xyz, Z = mol.atom_table()
    xyz_d = torch.as_tensor(xyz, device=dev)
    Z_d = torch.as_tensor(Z, device=dev)
    g = torch.zeros(mol.natom * 3, dtype=torch.float64, device=dev)
    prec = _lib.PRECISION[precision or fb.precision]
    with torch.cuda.device(dev):
        st = _stream_ptr()
        _lib.check(L.sf_grad_one_electron(fb.handle, _ptr(xyz_d), _ptr(Z_d), mol.natom, _ptr(D), _ptr(W), _ptr(g),
                                          st))
        _lib.check(L.sf_grad_jk(fb.handle, _ptr(D), _ptr(g), prec, fb.cutoff if cutoff is None else cutoff,
                                fb.fp32_cutoff if fp32_cutoff is None else fp32_cutoff, st))
    g = g.view(mol.natom, 3) + torch.as_tensor(nuclear_repulsion_gradient(mol), device=dev)
    return g


class RHFEnergy(torch.autograd.Function):
    """E_RHF(coords) with analytic forces in backward.

    ``RHFEnergy.apply(coords_bohr, symbols, basis, options)``: coords is an
    (natom, 3) float64 tensor in bohr; options a dict of scf_diis keywords
    (precision, cutoff, fp32_cutoff, tol, dtol) -- the same precision is used
    for the backward pass."""

    @staticmethod
    def forward(ctx, coords, symbols, basis, options=None):
        opts = dict(options or {})
        precision = opts.pop("precision", "fp64")
        cutoff = opts.pop("cutoff", 1e-12)
        fp32_cutoff = opts.pop("fp32_cutoff", 1e-2)
        opts.setdefault("tol", 1e-10)
        opts.setdefault("dtol", 1e-8)
        dev = coords.device if coords.is_cuda else torch.device("cuda")
        mol = Molecule.from_geometry(list(symbols), coords.detach().cpu().numpy() * BOHR, basis)
        fb = FockBuilder(mol, device=dev, cutoff=cutoff, fp32_cutoff=fp32_cutoff, precision=precision)
        res = scf_diis(mol, fb=fb, device=dev, **opts)
        ctx.state = (mol, res, fb, precision)
        ctx.coords_device = coords.device
        return torch.tensor(res.energy, dtype=torch.float64, device=coords.device)

    @staticmethod
    def backward(ctx, grad_out):
        mol, res, fb, precision = ctx.state
        g = rhf_gradient(mol, res, fb, precision=precision)
        fb.close()
        ctx.state = None
        return grad_out * g.to(ctx.coords_device), None, None, None


def energy_and_forces(symbols, coords_bohr, basis, **options):
    """Convenience: (E, F = -dE/dR) for a geometry in bohr."""
    x = torch.tensor(np.asarray(coords_bohr, dtype=np.float64), requires_grad=True)
    E = RHFEnergy.apply(x, tuple(symbols), basis, options)
    E.backward()
    return float(E), -x.grad.numpy()
