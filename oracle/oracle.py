"""CPU ORACLE (test infrastructure only) -- Python side.

Only tests/, the smoke check in __graft_entry__.py and the cpu_baseline /
reference legs of bench.py may import this module; the product path never does.

It loads ``oracle/liboracle.so`` (a C restatement of the reference's integral
engine, see rys_oracle.c) and adds the reference's Python-level drivers:

* ``build_eri_dense``  hf.py:33-61 (unique quartets, 8-fold scatter, dense N^4)
* ``jk_dense``         hf.py:300   (G = einsum(pqrs,rs) - 1/2 einsum(prqs,rs))
* ``jk_direct``        the same J/K from the unique quartets without the tensor
* ``scf_diis``         hf.py:237-353 (Loewdin, eigh, cDIIS with 7 vectors max,
                       DIIS from iteration 3, |dE| <= tol)
* ``one_electron``     mmd.py:32-141 + hf.py:266-274 (S, T, V)

``use_reference_root5()`` swaps the oracle's own root generator for the
reference's root5 fits transcribed into oracle/_ref/ (see gen_ref_root5.py).
"""
from __future__ import annotations

import ctypes as C
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB = os.path.join(HERE, "liboracle.so")
REF_LIB = os.path.join(HERE, "_ref", "librefroot5.so")
MAXK = 16


def build(force: bool = False) -> str:
    """Compile the C restatement (gcc -O2, OpenMP, no fast-math)."""
    src = os.path.join(HERE, "rys_oracle.c")
    if force or not os.path.exists(LIB) or os.path.getmtime(LIB) < os.path.getmtime(src):
        subprocess.check_call(["gcc", "-O2", "-fopenmp", "-shared", "-fPIC", "-o", LIB, src, "-lm"])
    return LIB


class CGF(C.Structure):
    _fields_ = [("K", C.c_int), ("shell", C.c_int * 3), ("center", C.c_double * 3),
                ("expns", C.c_double * MAXK), ("coefs", C.c_double * MAXK), ("nf", C.c_double * MAXK)]


_lib = None
_ref = None


def lib():
    global _lib
    if _lib is None:
        build()
        _lib = C.CDLL(LIB)
        d, i, p = C.c_double, C.c_int, C.c_void_p
        _lib.orc_boys.restype = d
        _lib.orc_boys.argtypes = [i, d]
        _lib.orc_rys_roots_exact.argtypes = [i, d, p, p]
        _lib.orc_root5.argtypes = [d, p]
        _lib.orc_set_root_mode.argtypes = [i, p]
        _lib.orc_eri_rys.restype = d
        _lib.orc_eri_rys.argtypes = [p, p, p, p]
        _lib.orc_mmd_eri.restype = d
        _lib.orc_mmd_eri.argtypes = [p, p, p, p]
        _lib.orc_hermite_e.restype = d
        _lib.orc_hermite_e.argtypes = [i, i, i, d, d, d]
        _lib.orc_coulomb_r.restype = d
        _lib.orc_coulomb_r.argtypes = [i, i, i, i, d, d, d, d, d]
        _lib.orc_eri_list.argtypes = [p, p, C.c_int64, p, i, i]
        _lib.orc_build_eri_dense.argtypes = [p, i, p, i, i]
        _lib.orc_jk_direct.argtypes = [p, i, p, p, p, i, i, C.c_int64, C.c_int64]
        _lib.orc_one_electron.argtypes = [p, i, p, p, i, p, p, p, i]
        _lib.orc_num_unique.restype = C.c_int64
        _lib.orc_num_unique.argtypes = [i]
        _lib.orc_max_threads.restype = i
        _lib.orc_init()
    return _lib


def have_reference_root5() -> bool:
    return os.path.exists(REF_LIB)


def use_reference_root5(on: bool = True) -> bool:
    """Route the oracle's 5-root evaluation through the reference's root5 fits."""
    global _ref
    L = lib()
    if not on:
        L.orc_set_root_mode(0, None)
        return False
    if not have_reference_root5():
        return False
    if _ref is None:
        _ref = C.CDLL(REF_LIB)
    fn = C.cast(_ref.ref_root5, C.c_void_p)
    L.orc_set_root_mode(2, fn)
    return True


def use_exact_roots(on: bool = True):
    lib().orc_set_root_mode(1 if on else 0, None)


def ref_root5(x: float) -> np.ndarray:
    global _ref
    if _ref is None:
        _ref = C.CDLL(REF_LIB)
        _ref.ref_root5.argtypes = [C.c_void_p, C.c_void_p]
    xx = np.array([x], dtype=np.float64)
    out = np.zeros(10)
    _ref.ref_root5(xx.ctypes.data, out.ctypes.data)
    return out


def boys(m: int, x: float) -> float:
    return lib().orc_boys(m, x)


def rys_roots_exact(n: int, x: float):
    u = np.zeros(n)
    w = np.zeros(n)
    lib().orc_rys_roots_exact(n, float(x), u.ctypes.data, w.ctypes.data)
    return u, w


def root5(x: float) -> np.ndarray:
    out = np.zeros(10)
    lib().orc_root5(float(x), out.ctypes.data)
    return out


def make_cgf(coefs, expns, shell, nf, center) -> CGF:
    c = CGF()
    K = len(coefs)
    if K > MAXK:
        raise ValueError("contraction too long for the oracle")
    c.K = K
    for d in range(3):
        c.shell[d] = int(shell[d])
        c.center[d] = float(center[d])
    for k in range(K):
        c.coefs[k] = float(coefs[k])
        c.expns[k] = float(expns[k])
        c.nf[k] = float(nf[k])
    return c


def cgf_array(cgfs):
    """Reference-style CGF objects (coefs, expns, shell, normalize_factors, center) -> C array."""
    arr = (CGF * len(cgfs))()
    for i, g in enumerate(cgfs):
        arr[i] = make_cgf(g.coefs, g.expns, g.shell, g.normalize_factors, g.center)
    return arr


def eri_rys(c1, c2, c3, c4, e1, e2, e3, e4, s1, s2, s3, s4, n1, n2, n3, n4, r1, r2, r3, r4) -> float:
    """Same 20 arguments as rys.eri_rys (core.f90:967-975, hf.py:26-30)."""
    a = make_cgf(c1, e1, s1, n1, r1)
    b = make_cgf(c2, e2, s2, n2, r2)
    c = make_cgf(c3, e3, s3, n3, r3)
    d = make_cgf(c4, e4, s4, n4, r4)
    return lib().orc_eri_rys(C.byref(a), C.byref(b), C.byref(c), C.byref(d))


def eri_mmd(g1, g2, g3, g4) -> float:
    a, b, c, d = (make_cgf(g.coefs, g.expns, g.shell, g.normalize_factors, g.center) for g in (g1, g2, g3, g4))
    return lib().orc_mmd_eri(C.byref(a), C.byref(b), C.byref(c), C.byref(d))


def eri_list(cgfs, idx, method: str = "rys", nthreads: int = 0) -> np.ndarray:
    arr = cgf_array(cgfs) if not isinstance(cgfs, C.Array) else cgfs
    idx = np.ascontiguousarray(idx, dtype=np.int32).reshape(-1, 4)
    out = np.zeros(len(idx))
    lib().orc_eri_list(C.cast(arr, C.c_void_p), idx.ctypes.data, len(idx), out.ctypes.data,
                       1 if method == "mmd" else 0, nthreads)
    return out


def build_eri_dense(cgfs, method: str = "rys", nthreads: int = 0) -> np.ndarray:
    n = len(cgfs)
    arr = cgf_array(cgfs)
    out = np.zeros((n, n, n, n))
    lib().orc_build_eri_dense(C.cast(arr, C.c_void_p), n, out.ctypes.data, 1 if method == "mmd" else 0, nthreads)
    return out


def jk_dense(eri: np.ndarray, P: np.ndarray):
    """hf.py:300 digestion: J = einsum(pqrs,rs), K = einsum(prqs,rs); G = J - K/2."""
    J = np.einsum("pqrs,rs->pq", eri, P, optimize=True)
    K = np.einsum("prqs,rs->pq", eri, P, optimize=True)
    return J, K


def jk_direct(cgfs, D: np.ndarray, method: str = "rys", nthreads: int = 0, stride: int = 1, phase: int = 0):
    n = len(cgfs)
    arr = cgf_array(cgfs) if not isinstance(cgfs, C.Array) else cgfs
    D = np.ascontiguousarray(D, dtype=np.float64)
    J = np.zeros((n, n))
    K = np.zeros((n, n))
    lib().orc_jk_direct(C.cast(arr, C.c_void_p), n, D.ctypes.data, J.ctypes.data, K.ctypes.data,
                        1 if method == "mmd" else 0, nthreads, stride, phase)
    return J, K


def one_electron(cgfs, atom_xyz_bohr, charges, nthreads: int = 0):
    n = len(cgfs)
    arr = cgf_array(cgfs)
    xyz = np.ascontiguousarray(atom_xyz_bohr, dtype=np.float64)
    Z = np.ascontiguousarray(charges, dtype=np.float64)
    S = np.zeros((n, n)); T = np.zeros((n, n)); V = np.zeros((n, n))
    lib().orc_one_electron(C.cast(arr, C.c_void_p), n, xyz.ctypes.data, Z.ctypes.data, len(Z),
                           S.ctypes.data, T.ctypes.data, V.ctypes.data, nthreads)
    return S, T, V


def num_unique(n: int) -> int:
    return lib().orc_num_unique(n)


def scf_diis(S, T, V, nelec: int, e_nuc: float, jk, tol: float = 1e-10, maxiter: int = 100):
    """hf.py:237-353 restated.  ``jk(P) -> (J, K)``.  Returns (E_total, P, F, niter)."""
    H = T + V
    vals, vecs = np.linalg.eigh(S)
    X = vecs @ np.diag(1.0 / np.sqrt(vals)) @ vecs.T
    norb = nelec // 2
    F = H.copy()
    Fs, res = [], []
    etot_old = float("inf")
    counter = 0
    P = None
    while True:
        e, Cp = np.linalg.eigh(X @ F @ X)
        Cm = X @ Cp
        Co = Cm[:, :norb]
        P = 2.0 * Co @ Co.T
        J, K = jk(P)
        F = H + J - 0.5 * K
        etot = 0.5 * np.sum(P * (H + F))
        if abs(etot - etot_old) <= tol:
            break
        counter += 1
        etot_old = etot
        if counter > maxiter:
            break
        if counter <= 2:
            continue
        if len(Fs) > 6:
            Fs.pop(0)
            res.pop(0)
        res.append(X @ (F @ P @ S - S @ P @ F) @ X)
        Fs.append(F)
        nb = len(Fs) + 1
        B = np.zeros((nb, nb))
        B[-1, :] = -1.0
        B[:, -1] = -1.0
        B[-1, -1] = 0.0
        for i in range(len(Fs)):
            for j in range(len(Fs)):
                B[i, j] += np.trace(res[i].T @ res[j])
        rhs = np.zeros(nb)
        rhs[-1] = -1.0
        try:
            cc = np.linalg.solve(B, rhs)
        except np.linalg.LinAlgError:
            continue
        F = np.zeros_like(F)
        for i in range(len(cc) - 1):
            F += Fs[i] * cc[i]
    return etot + e_nuc, P, F, counter
