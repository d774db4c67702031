"""RHF with the SCF iteration captured as one CUDA graph.

Same iteration as scf_diis (src/hf/hf.py:237-353): density from the current
Fock matrix, Fock build F = H + J - K/2, energy 1/2 sum P(H+F), convergence
when |dE| <= tol, Pulay cDIIS with error X(FPS - SPF)X, at most 7 vectors,
from the third iteration, a singular Pulay system keeps the plain F.  What
changes is how each step is made free of host synchronisation, so that the
whole iteration replays as a single graph launch:

* density: instead of eigh (which reports its status to the host), the
  projector onto the lowest nocc eigenvectors of F' = X F X is obtained by
  trace-correcting purification (Niklasson's TC2): X0 = (e_max - F')/(e_max -
  e_min) with Gershgorin bounds, then a fixed number of steps X <- X^2 or
  2X - X^2, the branch chosen on the device by comparing traces; D = 2 X P X.
  At convergence this is the same density as diagonalisation.
* DIIS: a fixed ring of 7 Fock/error matrices with a validity mask; unused
  slots get unit diagonal and zero coupling in the bordered Pulay matrix, so
  their coefficients vanish; the system is solved on the device
  (sf_small_solve); a singular system or an iteration before the third
  selects the plain F on the device.
* Fock build: FockBuilder.jk into static buffers (the library launches its
  class kernels on streams forked from the capturing stream).
The host replays the graph once per iteration and reads dE from pinned
memory; convergence is checked exactly as in the reference.  Where torch
keeps the captured graph (CUDAGraph(keep_graph=True)) the library
instantiates it with node priorities (sf_graph_instantiate), so the Fock
build's accurate tier keeps its high-priority side streams on replay.
"""
from __future__ import annotations

import ctypes as C

import torch

from . import _lib
from .fock import FockBuilder
from .molecule import Molecule
from .scf import SCFResult, preload_torch_linalg

NSLOT = 7          # DIIS vectors kept (hf.py:291, 324-326)


class GraphSCF:
    def __init__(self, mol: Molecule, fb: FockBuilder | None = None, precision: str = "fp64",
                 cutoff: float = 1e-12, fp32_cutoff: float = 1e-2, purification_steps: int = 60,
                 device="cuda"):
        preload_torch_linalg()
        self.mol = mol
        self.fb = fb or FockBuilder(mol, device=device, cutoff=cutoff, fp32_cutoff=fp32_cutoff, precision=precision)
        self.precision = precision
        self.cutoff = cutoff
        self.fp32_cutoff = fp32_cutoff
        self.steps = purification_steps
        dev = self.fb.device
        self.dev = dev
        S, T, V = self.fb.one_electron()
        self.S, self.H = S, T + V
        vals, vecs = torch.linalg.eigh(S)
        self.X = (vecs @ torch.diag(1.0 / torch.sqrt(vals)) @ vecs.T).contiguous()
        n = self.fb.nao
        self.n = n
        self.nocc = mol.nelectron // 2
        z = lambda *s: torch.zeros(*s, dtype=torch.float64, device=dev)
        self.F = self.H.clone()
        self.Fnew = z(n, n)
        self.D = z(n, n)
        self.J, self.K = z(n, n), z(n, n)
        self.E = z(())
        self.Eold = torch.full((), float("inf"), dtype=torch.float64, device=dev)
        self.dE = z(())
        self.count = z(())            # iterations done (hf.py: counter)
        self.Fs = z(NSLOT, n, n)
        self.Rs = z(NSLOT, n, n)
        self.mask = z(NSLOT)
        self.slot = z(())             # next ring slot
        self.B = z(NSLOT + 1, NSLOT + 1)
        self.rhs = z(NSLOT + 1)
        self.rhs[-1] = -1.0
        self.coef = z(NSLOT + 1)
        self.ok = z(())
        self.eye = torch.eye(n, dtype=torch.float64, device=dev)
        self.slots = torch.arange(NSLOT, dtype=torch.float64, device=dev)
        self.dE_host = torch.zeros((), dtype=torch.float64).pin_memory()
        self.graph = None
        self._exec = None

    # ------------------------------------------------------------------
    def _purify(self, Fp):
        """Projector onto the nocc lowest eigenvectors of Fp (TC2)."""
        n, nocc = self.n, float(self.nocc)
        d = torch.diagonal(Fp)
        r = Fp.abs().sum(dim=1) - d.abs()
        emin = torch.min(d - r)
        emax = torch.max(d + r)
        Xp = (emax * self.eye - Fp) / (emax - emin)
        for _ in range(self.steps):
            X2 = Xp @ Xp
            tr, tr2 = torch.trace(Xp), torch.trace(X2)
            w = (torch.abs(tr2 - nocc) < torch.abs(2.0 * tr - tr2 - nocc)).to(torch.float64)
            Xp = w * X2 + (1.0 - w) * (2.0 * Xp - X2)
        return Xp

    def _iteration(self):
        L = _lib.lib()
        X, H, S = self.X, self.H, self.S
        Pp = self._purify(X @ self.F @ X)
        self.D.copy_(2.0 * X @ Pp @ X)
        self.fb.jk(self.D, precision=self.precision, cutoff=self.cutoff, fp32_cutoff=self.fp32_cutoff,
                   out=(self.J, self.K))
        self.Fnew.copy_(H + self.J - 0.5 * self.K)
        self.E.copy_(0.5 * torch.sum(self.D * (H + self.Fnew)))
        self.dE.copy_(self.E - self.Eold)
        self.Eold.copy_(self.E)
        self.count.add_(1.0)
        # DIIS (applied from the third iteration on, hf.py:317-319)
        use = (self.count > 2.0).to(torch.float64)
        Rn = X @ (self.Fnew @ self.D @ S - S @ self.D @ self.Fnew) @ X
        onehot = (self.slots == self.slot).to(torch.float64) * use
        keep = 1.0 - onehot
        self.Fs.mul_(keep.view(-1, 1, 1)).add_(onehot.view(-1, 1, 1) * self.Fnew)
        self.Rs.mul_(keep.view(-1, 1, 1)).add_(onehot.view(-1, 1, 1) * Rn)
        self.mask.copy_(torch.clamp(self.mask + onehot, max=1.0))
        self.slot.copy_(torch.remainder(self.slot + use, float(NSLOT)))
        G = torch.einsum("iab,jab->ij", self.Rs, self.Rs)
        m = self.mask
        Bm = G * torch.outer(m, m) + torch.diag(1.0 - m)
        # bordered Pulay matrix assembled on the device (an item assignment of
        # a Python number would copy from the host, which capture forbids)
        top = torch.cat([Bm, -m.view(-1, 1)], dim=1)
        bottom = torch.cat([-m.view(1, -1), torch.zeros(1, 1, dtype=m.dtype, device=m.device)], dim=1)
        self.B.copy_(torch.cat([top, bottom], dim=0))
        _lib.check(L.sf_small_solve(NSLOT + 1, C.c_void_p(self.B.data_ptr()), C.c_void_p(self.rhs.data_ptr()),
                                    C.c_void_p(self.coef.data_ptr()), C.c_void_p(self.ok.data_ptr()),
                                    C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        Fd = torch.einsum("i,iab->ab", self.coef[:NSLOT] * m, self.Fs)
        sel = use * self.ok
        self.F.copy_(sel * Fd + (1.0 - sel) * self.Fnew)

    # ------------------------------------------------------------------
    def capture(self):
        """Warm up (builds the quartet lists, cuBLAS handles) and capture."""
        if self._exec is not None:
            _lib.lib().sf_fock_graph_destroy(self._exec)
            self._exec = None
        state = [t.clone() for t in (self.F, self.Eold, self.count, self.Fs, self.Rs, self.mask, self.slot)]
        s = torch.cuda.Stream(device=self.dev)
        s.wait_stream(torch.cuda.current_stream())
        with torch.cuda.stream(s):
            for _ in range(2):
                self._iteration()
        torch.cuda.current_stream().wait_stream(s)
        for t, v in zip((self.F, self.Eold, self.count, self.Fs, self.Rs, self.mask, self.slot), state):
            t.copy_(v)
        torch.cuda.synchronize()
        # keep the captured cudaGraph_t where torch allows it and instantiate it
        # through the library with node priorities: replayed by torch, every
        # node runs at the launching stream's priority and the Fock build's
        # accurate tier loses the high-priority side streams it has eagerly
        try:
            self.graph = torch.cuda.CUDAGraph(keep_graph=True)
            keep = True
        except TypeError:
            self.graph = torch.cuda.CUDAGraph()
            keep = False
        with torch.cuda.graph(self.graph):
            self._iteration()
        torch.cuda.synchronize()
        self._exec = None
        if keep:
            h = C.c_void_p()
            _lib.check(_lib.lib().sf_graph_instantiate(C.c_void_p(int(self.graph.raw_cuda_graph())), 1, C.byref(h)))
            self._exec = h
        return self

    def _replay(self):
        if self._exec is not None:
            _lib.check(_lib.lib().sf_fock_graph_launch(self._exec,
                                                       C.c_void_p(torch.cuda.current_stream().cuda_stream)))
        else:
            self.graph.replay()

    def __del__(self):
        ex = getattr(self, "_exec", None)
        if ex is not None:
            try:
                _lib.lib().sf_fock_graph_destroy(ex)
            except Exception:
                pass
            self._exec = None

    def run(self, tol: float = 1e-8, maxiter: int = 100) -> SCFResult:
        if self.graph is None:
            self.capture()
        converged = False
        it = 0
        hist = []
        while True:
            self._replay()
            self.dE_host.copy_(self.dE, non_blocking=True)
            torch.cuda.current_stream().synchronize()
            hist.append(float(self.E) + self.mol.e_nuc)
            if abs(float(self.dE_host)) <= tol:
                converged = True
                break
            it += 1
            if it > maxiter:
                break
        e = float(self.E)
        return SCFResult(energy=e + self.mol.e_nuc, e_elec=e, e_nuc=self.mol.e_nuc, iterations=it,
                         converged=converged, D=self.D.clone(), F=self.Fnew.clone(), C=None, eps=None,
                         H=self.H, S=self.S, history=hist)

    def replay_once(self):
        self._replay()


def scf_graph(mol: Molecule, tol=1e-8, maxiter=100, precision="fp64", cutoff=1e-12, fp32_cutoff=1e-2, fb=None,
              device="cuda", purification_steps=60) -> SCFResult:
    """scf_diis with every iteration one CUDA-graph replay."""
    g = GraphSCF(mol, fb=fb, precision=precision, cutoff=cutoff, fp32_cutoff=fp32_cutoff,
                 purification_steps=purification_steps, device=device)
    return g.run(tol=tol, maxiter=maxiter)
