"""The GPU Fock build behind the reference's ERI/Fock boundary.

Reference boundary (src/hf/hf.py):
* ``rys.eri_rys(...)`` per unique AO quartet (hf.py:26-30, core.f90:967-1002)
* ``build_eri_parallel(cgfs, ncgf)`` -> dense (N,N,N,N) tensor (hf.py:33-61)
* ``G = einsum('pqrs,rs') - 0.5 einsum('prqs,rs')`` each SCF iteration (hf.py:300)

Here:
* ``FockBuilder(mol).jk(D) -> (J, K)``: direct, Schwarz-screened J/K on the
  GPU (G = J - K/2), no N^4 tensor.  FP64, FP32 or mixed precision.
* ``FockBuilder(mol).build_eri()``: the dense tensor of build_eri_parallel,
  from the same GPU integrals (small molecules only: N^4 doubles).
* ``eri_rys(c1..c4, e1..e4, s1..s4, n1..n4, r1..r4)``: the 20-argument call of
  rys.eri_rys, evaluated by the GPU kernels.
* ``FockBuilder(mol).one_electron() -> (S, T, V)`` (hf.py:266-274).
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .molecule import Molecule

DEFAULT_CUTOFF = 1e-12        # Schwarz cutoff on Q_ab Q_cd
DEFAULT_FP32_CUTOFF = 1e-5    # mixed precision: Q_ab Q_cd below this run in FP32


def _stream_ptr(stream=None):
    s = stream if stream is not None else torch.cuda.current_stream()
    return C.c_void_p(s.cuda_stream)


def _ptr(t: torch.Tensor):
    return C.c_void_p(t.data_ptr())


def shell_descs(table: dict):
    """Shell table (Molecule.shell_table) -> ctypes array; returns (array, keepalive)."""
    n = len(table["l"])
    arr = (_lib.ShellDesc * n)()
    exps = np.ascontiguousarray(table["exps"], dtype=np.float64)
    coefs = np.ascontiguousarray(table["coefs"], dtype=np.float64)
    for s in range(n):
        o = int(table["prim_offset"][s])
        d = arr[s]
        d.l = int(table["l"][s])
        d.nprim = int(table["nprim"][s])
        d.atom = int(table["atom"][s])
        d.ao_offset = int(table["ao_offset"][s])
        for k in range(3):
            d.center[k] = float(table["center"][s][k])
        d.exps = exps[o:].ctypes.data_as(C.POINTER(C.c_double))
        d.coefs = coefs[o:].ctypes.data_as(C.POINTER(C.c_double))
    return arr, (exps, coefs)


class FockBuilder:
    """Direct-SCF J/K builder for one molecule on the current CUDA device."""

    def __init__(self, mol: Molecule | dict, device: str | torch.device = "cuda", cutoff: float = DEFAULT_CUTOFF,
                 fp32_cutoff: float = DEFAULT_FP32_CUTOFF, precision: str = "fp64"):
        L = _lib.lib()
        self.device = torch.device(device)
        if self.device.type != "cuda":
            raise ValueError("FockBuilder needs a CUDA device")
        if self.device.index is None:
            self.device = torch.device("cuda", torch.cuda.current_device())
        self.mol = mol if isinstance(mol, Molecule) else None
        table = mol.shell_table() if isinstance(mol, Molecule) else mol
        self.table = table
        self.cutoff = cutoff
        self.fp32_cutoff = fp32_cutoff
        self.precision = precision
        arr, keep = shell_descs(table)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            torch.cuda.current_stream().synchronize()
            _lib.check(L.sf_create(C.cast(arr, C.c_void_p), len(arr), C.byref(h)))
        self._h = h
        del keep
        self.nao = L.sf_nao(h)
        self.nshell = len(table["l"])
        self.l = np.asarray(table["l"])
        self.ao_offset = np.asarray(table["ao_offset"])
        self.q = self.schwarz()
        self.last_stats = None

    # ------------------------------------------------------------------
    def close(self):
        if getattr(self, "_h", None):
            _lib.lib().sf_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def handle(self):
        return self._h

    def schwarz(self) -> np.ndarray:
        q = np.zeros((self.nshell, self.nshell))
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().sf_schwarz(self._h, q.ctypes.data, _stream_ptr()))
        return q

    def set_density_screening(self, fock: bool = False, grad: bool = True, fock_fp32_cutoff: float = -1.0,
                              grad_drop_cutoff: float = -1.0, grad_fp32_cutoff: float = -1.0):
        """Density-weighted classification of every later Fock build and
        gradient (sf_set_density_screening).  ``fock``: the mixed modes run an
        accurate-tier quartet in FP32 when its density-weighted bound is below
        the FP32 cutoff (off by default: the split then follows D between SCF
        iterations and slows convergence).  ``grad``: the gradient leaves out
        quartets whose bound is below the drop cutoff (on by default).
        Negative cutoffs: the call's own."""
        flags = (1 if fock else 0) | (2 if grad else 0)
        _lib.check(_lib.lib().sf_set_density_screening(self._h, flags, fock_fp32_cutoff,
                                                       grad_drop_cutoff, grad_fp32_cutoff))

    def set_launch_mode(self, mode: str = "streams", ctas_per_sm: int = 0):
        """How Fock builds launch their class kernels (sf_set_launch_mode):
        "streams" (one launch per class slice on 16 side streams) or
        "persistent" (the FP32 register-path classes as one persistent launch
        per register tier, fed by a device work queue)."""
        m = {"streams": 0, "persistent": 1}[mode]
        _lib.check(_lib.lib().sf_set_launch_mode(self._h, m, ctas_per_sm))

    def set_partition(self, part: int, nparts: int):
        _lib.check(_lib.lib().sf_set_partition(self._h, part, nparts))

    # ------------------------------------------------------------------
    def jk(self, D: torch.Tensor, precision: str | None = None, cutoff: float | None = None,
           fp32_cutoff: float | None = None, out=None, stats: bool = False):
        """J_pq = sum (pq|rs) D_rs and K_pq = sum (pr|qs) D_rs for symmetric D."""
        prec = _lib.PRECISION[precision or self.precision]
        n = self.nao
        if D.shape != (n, n) or D.dtype != torch.float64 or D.device != self.device:
            raise ValueError("D must be a (%d,%d) float64 tensor on %s" % (n, n, self.device))
        D = D.contiguous()
        if out is None:
            J = torch.empty((n, n), dtype=torch.float64, device=self.device)
            K = torch.empty((n, n), dtype=torch.float64, device=self.device)
        else:
            J, K = out
        st = _lib.Stats() if stats else None
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().sf_fock_jk(self._h, _ptr(D), _ptr(J), _ptr(K), prec,
                                             self.cutoff if cutoff is None else cutoff,
                                             self.fp32_cutoff if fp32_cutoff is None else fp32_cutoff,
                                             C.byref(st) if st is not None else None, _stream_ptr()))
        if st is not None:
            self.last_stats = st.as_dict()
        return J, K

    def capture_jk(self, D: torch.Tensor, J: torch.Tensor, K: torch.Tensor, precision: str | None = None,
                   native: bool = False, node_priority: bool = True):
        """Capture one Fock build J, K = jk(D) on these static tensors as a CUDA
        graph (the class launches and their stream fork/join become graph
        nodes); returns the graph -- ``g.replay()`` rebuilds J and K for the
        current contents of D without any host-side launch work.

        native=False: a torch.cuda.CUDAGraph (composable with torch ops in the
        same capture).  native=True: the library captures and instantiates the
        graph itself (sf_fock_jk_graph_create), with node_priority keeping each
        launch's side-stream priority on replay."""
        if native:
            for t in (D, J, K):
                if t.shape != (self.nao, self.nao) or t.dtype != torch.float64 or t.device != self.device \
                        or not t.is_contiguous():
                    raise ValueError("D, J, K must be contiguous (%d,%d) float64 tensors on %s"
                                     % (self.nao, self.nao, self.device))
            return _NativeFockGraph(self, D, J, K, _lib.PRECISION[precision or self.precision], node_priority)
        self.jk(D, precision=precision, out=(J, K))          # builds the quartet lists (allocates)
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            self.jk(D, precision=precision, out=(J, K))
        torch.cuda.synchronize()
        return g

    def autotune(self, D: torch.Tensor, precision: str | None = None, cutoff: float | None = None,
                 fp32_cutoff: float | None = None, reps: int = 3):
        """Time candidate primitive splits of every launch of a Fock build at
        these settings and keep the fastest (sf_autotune); returns the table."""
        prec = _lib.PRECISION[precision or self.precision]
        if D.shape != (self.nao, self.nao) or D.dtype != torch.float64 or D.device != self.device:
            raise ValueError("D must be a (%d,%d) float64 tensor on %s" % (self.nao, self.nao, self.device))
        D = D.contiguous()
        with torch.cuda.device(self.device):
            rc = _lib.lib().sf_autotune(self._h, _ptr(D), prec, self.cutoff if cutoff is None else cutoff,
                                        self.fp32_cutoff if fp32_cutoff is None else fp32_cutoff, int(reps),
                                        _stream_ptr())
        if rc < 0:
            _lib.check(rc)
        return self.tuning()

    def tuning(self):
        """The recorded launch splits: list of dicts (cls, precision, cost, split, ms_default, ms_tuned)."""
        L = _lib.lib()
        out = []
        for i in range(L.sf_tuning_count(self._h)):
            e = _lib.TuneEntry()
            _lib.check(L.sf_get_tuning(self._h, i, C.byref(e)))
            out.append(e.as_dict())
        return out

    def set_tuning(self, table):
        """Load a table returned by `tuning()` (e.g. read back from JSON)."""
        arr = (_lib.TuneEntry * max(len(table), 1))()
        for i, e in enumerate(table):
            arr[i] = _lib.TuneEntry(int(e["cls"]), int(e["precision"]), int(e["cost"]), int(e["split"]),
                                    float(e.get("ms_default", 0.0)), float(e.get("ms_tuned", 0.0)))
        _lib.check(_lib.lib().sf_set_tuning(self._h, arr, len(table)))

    def save_tuning(self, path: str):
        import json
        with open(path, "w") as f:
            json.dump({"nao": self.nao, "entries": self.tuning()}, f, indent=1)

    def load_tuning(self, path: str):
        import json
        with open(path) as f:
            self.set_tuning(json.load(f)["entries"])

    def set_profiling(self, on=True):
        """True/1: time every class launch; 2: also serialise the launches on
        the caller's stream so each time is the kernel alone."""
        _lib.check(_lib.lib().sf_set_profiling(self._h, int(on)))

    def slice_info(self):
        """Per-launch work and (when profiling) device time of the last Fock build."""
        L = _lib.lib()
        out = []
        for i in range(L.sf_slice_count(self._h)):
            si = _lib.SliceInfo()
            _lib.check(L.sf_get_slice_info(self._h, i, C.byref(si)))
            out.append(si.as_dict())
        return out

    def fock(self, H: torch.Tensor, D: torch.Tensor, **kw):
        """F = H + J - K/2 (hf.py:300-301)."""
        J, K = self.jk(D, **kw)
        return H + J - 0.5 * K

    # ------------------------------------------------------------------
    def eri_plan(self, quartets) -> "EriPlan":
        """Prepare a raw-ERI batch of shell quartets (nq,4) for repeated runs."""
        return EriPlan(self, quartets)

    def eri_quartets(self, quartets, precision: str = "fp64"):
        """Contracted integrals of shell quartets (nq,4): list of (na,nb,nc,nd) arrays."""
        q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
        nc = (self.l + 1) * (self.l + 2) // 2
        plan = self.eri_plan(q)
        try:
            flat = plan.run(precision).cpu().numpy()
            offs = plan.offsets
        finally:
            plan.close()
        sizes = np.prod(nc[q], axis=1).astype(np.int64)
        return [flat[o:o + s].reshape(tuple(nc[row])) for o, s, row in zip(offs, sizes, q)]

    def build_eri(self, precision: str = "fp64") -> np.ndarray:
        """Dense (N,N,N,N) tensor as build_eri_parallel (hf.py:33-61); small N only."""
        n = self.nao
        ns = self.nshell
        quartets = []
        for a in range(ns):
            for b in range(a + 1):
                for c in range(ns):
                    for d in range(c + 1):
                        if a * (a + 1) // 2 + b >= c * (c + 1) // 2 + d:
                            quartets.append((a, b, c, d))
        blocks = self.eri_quartets(np.array(quartets, dtype=np.int32), precision)
        E = np.zeros((n, n, n, n))
        o = self.ao_offset
        for (a, b, c, d), blk in zip(quartets, blocks):
            sa, sb, sc, sd = (slice(o[x], o[x] + blk.shape[k]) for k, x in enumerate((a, b, c, d)))
            E[sa, sb, sc, sd] = blk
            E[sb, sa, sc, sd] = blk.transpose(1, 0, 2, 3)
            E[sa, sb, sd, sc] = blk.transpose(0, 1, 3, 2)
            E[sb, sa, sd, sc] = blk.transpose(1, 0, 3, 2)
            E[sc, sd, sa, sb] = blk.transpose(2, 3, 0, 1)
            E[sd, sc, sa, sb] = blk.transpose(3, 2, 0, 1)
            E[sc, sd, sb, sa] = blk.transpose(2, 3, 1, 0)
            E[sd, sc, sb, sa] = blk.transpose(3, 2, 1, 0)
        return E

    # ------------------------------------------------------------------
    def one_electron(self, atom_xyz=None, charges=None):
        """S, T, V (hf.py:266-274); nuclei default to the molecule's atoms."""
        if atom_xyz is None:
            atom_xyz, charges = self.mol.atom_table()
        n = self.nao
        xyz = torch.as_tensor(np.ascontiguousarray(atom_xyz, dtype=np.float64), device=self.device)
        Z = torch.as_tensor(np.ascontiguousarray(charges, dtype=np.float64), device=self.device)
        S = torch.empty((n, n), dtype=torch.float64, device=self.device)
        T = torch.empty_like(S)
        V = torch.empty_like(S)
        with torch.cuda.device(self.device):
            _lib.check(_lib.lib().sf_one_electron(self._h, _ptr(xyz), _ptr(Z), len(Z), _ptr(S), _ptr(T), _ptr(V),
                                                  _stream_ptr()))
        return S, T, V


class EriPlan:
    """A raw-ERI batch (sf_eri_plan): the quartets are canonicalised, grouped
    by class and cost-sorted once; ``run`` evaluates all of them (FP64 or FP32,
    stored as float64) into one packed device vector, quartet q at
    ``offsets[q]`` in row-major (a, b, c, d) component order."""

    def __init__(self, fb: FockBuilder, quartets):
        q = np.ascontiguousarray(quartets, dtype=np.int32).reshape(-1, 4)
        self.fb = fb
        self.nq = len(q)
        h = C.c_void_p()
        with torch.cuda.device(fb.device):
            _lib.check(_lib.lib().sf_eri_plan_create(fb.handle, q.ctypes.data, self.nq, C.byref(h)))
        self._p = h
        outs, prims, flops = C.c_int64(), C.c_int64(), C.c_double()
        _lib.check(_lib.lib().sf_eri_plan_info(self._p, C.byref(outs), C.byref(prims), C.byref(flops)))
        self.outputs, self.prim_quartets, self.flop_alg = outs.value, prims.value, flops.value
        self.offsets = np.zeros(self.nq, dtype=np.int64)
        _lib.check(_lib.lib().sf_eri_plan_offsets(self._p, self.offsets.ctypes.data))

    def run(self, precision: str = "fp64", out: torch.Tensor | None = None, engine: str = "rys") -> torch.Tensor:
        """engine "rys" (production kernels) or "md" (McMurchie-Davidson: FP64 on the
        CUDA cores, or FP32 with the bra E contraction on the tensor cores)."""
        if precision not in ("fp64", "fp32", "df"):
            raise ValueError("precision must be fp64, fp32 or df")
        if engine not in ("rys", "md"):
            raise ValueError("engine must be rys or md")
        if out is None:
            out = torch.empty(max(self.outputs, 1), dtype=torch.float64, device=self.fb.device)
        elif out.dtype != torch.float64 or out.numel() < self.outputs or not out.is_contiguous():
            raise ValueError("out must be a contiguous float64 tensor of >= %d values" % self.outputs)
        fn = _lib.lib().sf_eri_plan_run if engine == "rys" else _lib.lib().sf_eri_plan_run_md
        with torch.cuda.device(self.fb.device):
            _lib.check(fn(self._p, _lib.PRECISION[precision], _ptr(out), _stream_ptr()))
        return out

    def close(self):
        if getattr(self, "_p", None):
            with torch.cuda.device(self.fb.device):
                _lib.lib().sf_eri_plan_destroy(self._p)
            self._p = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


def _comp_factor(shell) -> float:
    """Library factor of component (lx,ly,lz) relative to x^l (see segfock.h)."""
    from .molecule import factorial2
    l = sum(shell)
    return np.sqrt(factorial2(2 * l - 1) / (factorial2(2 * shell[0] - 1) * factorial2(2 * shell[1] - 1) *
                                            factorial2(2 * shell[2] - 1)))


def _comp_index(shell) -> int:
    from .molecule import CART
    return CART[sum(shell)].index(tuple(int(v) for v in shell))


def eri_rys(coefs1, coefs2, coefs3, coefs4, expns1, expns2, expns3, expns4, shell1, shell2, shell3, shell4,
            normalize_factors1, normalize_factors2, normalize_factors3, normalize_factors4,
            center1, center2, center3, center4, device="cuda") -> float:
    """Drop-in for ``rys.eri_rys`` (core.f90:967-1002; called at hf.py:26-30):
    one contracted Cartesian AO quartet, same 20 arguments and meaning, computed
    by the GPU kernels.  ``shell`` beyond l = 2 raises SegFockError."""
    args = [(coefs1, expns1, shell1, normalize_factors1, center1), (coefs2, expns2, shell2, normalize_factors2, center2),
            (coefs3, expns3, shell3, normalize_factors3, center3), (coefs4, expns4, shell4, normalize_factors4, center4)]
    ls, nprim, aoo, cen, exps, coefs, comp = [], [], [], [], [], [], []
    off = 0
    for c, e, s, nf, r in args:
        s = [int(v) for v in s]
        l = sum(s)
        if l > 2:
            raise _lib.SegFockError(-2, "eri_rys: angular momentum above d is not supported")
        eff = np.asarray(c, dtype=np.float64) * np.asarray(nf, dtype=np.float64) / _comp_factor(s)
        ls.append(l); nprim.append(len(eff)); aoo.append(off); cen.append(np.asarray(r, dtype=np.float64))
        exps.append(np.asarray(e, dtype=np.float64)); coefs.append(eff); comp.append(_comp_index(s))
        off += (l + 1) * (l + 2) // 2
    po = np.zeros(5, dtype=np.int32)
    po[1:] = np.cumsum(nprim)
    table = dict(l=np.array(ls, dtype=np.int32), nprim=np.array(nprim, dtype=np.int32),
                 atom=np.arange(4, dtype=np.int32), ao_offset=np.array(aoo, dtype=np.int32),
                 center=np.array(cen), prim_offset=po, exps=np.concatenate(exps), coefs=np.concatenate(coefs))
    fb = FockBuilder(table, device=device)
    try:
        blk = fb.eri_quartets(np.array([[0, 1, 2, 3]], dtype=np.int32))[0]
    finally:
        fb.close()
    return float(blk[comp[0], comp[1], comp[2], comp[3]])


class _NativeFockGraph:
    """A Fock build captured and instantiated by the library (see
    FockBuilder.capture_jk(native=True)); replay() launches it on the current
    stream, close() frees it."""

    def __init__(self, fb: "FockBuilder", D, J, K, prec: int, node_priority: bool):
        self._keep = (fb, D, J, K)
        self._g = C.c_void_p()
        with torch.cuda.device(fb.device):
            _lib.check(_lib.lib().sf_fock_jk_graph_create(fb.handle, _ptr(D), _ptr(J), _ptr(K), prec, fb.cutoff,
                                                          fb.fp32_cutoff, 1 if node_priority else 0, _stream_ptr(),
                                                          C.byref(self._g)))

    def replay(self):
        _lib.check(_lib.lib().sf_fock_graph_launch(self._g, _stream_ptr()))

    def close(self):
        if self._g:
            _lib.lib().sf_fock_graph_destroy(self._g)
            self._g = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
