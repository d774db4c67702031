"""Seeded synthetic molecules for the benchmark and parity workloads.

* ``water()``            H2O, O (0,0,0), H (+-0.757, 0.587, 0) Angstrom.
* ``water_cluster(n)``   (H2O)_n: the water monomer rotated by a uniform
                         random rotation about O, O on a 3.0 A cubic grid
                         (2x2x2 for n <= 8, 2x2x4 for n <= 16, in grid order)
                         plus uniform +-0.3 A jitter per coordinate;
                         numpy.random.default_rng(seed).
* ``alkane(nc)``         all-trans CnH2n+2 zig-zag chain: C-C 1.54 A, C-H
                         1.09 A, tetrahedral angles, uniform +-0.05 A noise.
* ``random_quartet_shells`` shells for the raw-ERI stress test: K in 1..6,
                         exponents log-uniform in [0.05, 1e4], coefficients
                         normalised as molecule.py:210-226, centres uniform in
                         a 10 A box.
All coordinates are returned in Angstrom (symbols, (n,3) array).
"""
from __future__ import annotations

import numpy as np

WATER = (["O", "H", "H"], np.array([[0.0, 0.0, 0.0], [0.757, 0.587, 0.0], [-0.757, 0.587, 0.0]]))


def water():
    return list(WATER[0]), WATER[1].copy()


def random_rotation(rng) -> np.ndarray:
    """Uniform random rotation matrix from a uniform unit quaternion."""
    u1, u2, u3 = rng.random(3)
    q = np.array([np.sqrt(1 - u1) * np.sin(2 * np.pi * u2), np.sqrt(1 - u1) * np.cos(2 * np.pi * u2),
                  np.sqrt(u1) * np.sin(2 * np.pi * u3), np.sqrt(u1) * np.cos(2 * np.pi * u3)])
    x, y, z, w = q
    return np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                     [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                     [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])


def water_cluster(n: int = 8, seed: int = 0, spacing: float = 3.0, jitter: float = 0.3):
    rng = np.random.default_rng(seed)
    dims = (2, 2, 2) if n <= 8 else (2, 2, 4) if n <= 16 else (3, 3, int(np.ceil(n / 9)))
    grid = [(i, j, k) for i in range(dims[0]) for j in range(dims[1]) for k in range(dims[2])][:n]
    syms, xyz = [], []
    for g in grid:
        R = random_rotation(rng)
        o = np.array(g, dtype=float) * spacing + rng.uniform(-jitter, jitter, 3)
        for s, r in zip(*WATER):
            syms.append(s)
            xyz.append(o + R @ r)
    return syms, np.array(xyz)


def alkane(nc: int = 20, seed: int = 0, noise: float = 0.05, rcc: float = 1.54, rch: float = 1.09):
    theta = np.deg2rad(109.47)
    c = np.zeros((nc, 3))
    for i in range(nc):
        c[i] = [i * rcc * np.sin(theta / 2), (i % 2) * rcc * np.cos(theta / 2), 0.0]
    zax = np.array([0.0, 0.0, 1.0])
    syms, xyz = ["C"] * nc, [x for x in c]
    for i in range(nc):
        if 0 < i < nc - 1:
            u = (c[i] - c[i - 1]) + (c[i] - c[i + 1])
            u /= np.linalg.norm(u)
            for s in (1, -1):
                d = u * np.cos(theta / 2) + s * zax * np.sin(theta / 2)
                syms.append("H")
                xyz.append(c[i] + rch * d)
        else:
            nb = c[1] - c[0] if i == 0 else c[nc - 2] - c[nc - 1]
            b = nb / np.linalg.norm(nb)
            e1 = np.cross(zax, b)
            e1 /= np.linalg.norm(e1)
            if i == 0:
                e1 = -e1 if np.dot(e1, c[2] - c[1]) > 0 else e1
            else:
                e1 = -e1 if np.dot(e1, c[nc - 3] - c[nc - 2]) > 0 else e1
            e2 = np.cross(b, e1)
            for k in range(3):
                ph = 2 * np.pi * k / 3
                d = -b / 3.0 + np.sqrt(8.0 / 9.0) * (np.cos(ph) * e1 + np.sin(ph) * e2)
                syms.append("H")
                xyz.append(c[i] + rch * d)
    rng = np.random.default_rng(seed)
    xyz = np.array(xyz) + rng.uniform(-noise, noise, (len(xyz), 3))
    return syms, xyz


def random_quartet_shells(nshell: int, seed: int = 0, lmax: int = 2, kmax: int = 6, box: float = 10.0):
    """Shell table (as Molecule.shell_table) of random normalised contracted shells."""
    from .molecule import BOHR, factorial2
    rng = np.random.default_rng(seed)
    ls = rng.integers(0, lmax + 1, nshell).astype(np.int32)
    nprim = rng.integers(1, kmax + 1, nshell).astype(np.int32)
    exps, coefs, cen = [], [], []
    for s in range(nshell):
        l, K = int(ls[s]), int(nprim[s])
        e = np.exp(rng.uniform(np.log(0.05), np.log(1e4), K))
        c = rng.uniform(0.1, 1.0, K)
        # primitive norms of the x^l component and contracted renormalisation (molecule.py:210-226)
        nf = np.sqrt(2.0 ** (2 * l + 1.5) * e ** (l + 1.5) / factorial2(2 * l - 1) / np.pi ** 1.5)
        pre = np.pi ** 1.5 * factorial2(2 * l - 1) / 2.0 ** l
        N = pre * np.sum(np.outer(nf * c, nf * c) / np.add.outer(e, e) ** (l + 1.5))
        exps.append(e)
        coefs.append(c * nf / np.sqrt(N))
        cen.append(rng.uniform(0, box, 3) / BOHR)
    nc = (ls + 1) * (ls + 2) // 2
    ao = np.zeros(nshell, dtype=np.int32)
    ao[1:] = np.cumsum(nc)[:-1]
    po = np.zeros(nshell + 1, dtype=np.int32)
    po[1:] = np.cumsum(nprim)
    return dict(l=ls, nprim=nprim, atom=np.arange(nshell, dtype=np.int32), ao_offset=ao,
                center=np.array(cen), prim_offset=po, exps=np.concatenate(exps), coefs=np.concatenate(coefs))


PAIR_L = [(0, 0), (1, 0), (1, 1), (2, 0), (2, 1), (2, 2)]
QUARTET_CLASSES = [(PAIR_L[x], PAIR_L[y]) for x in range(6) for y in range(x + 1)]


def random_quartet_batch(nq: int, nshell: int = 600, seed: int = 0, kmax: int = 6, box: float = 10.0):
    """Raw-ERI stress batch: a pool of `nshell` random shells
    (random_quartet_shells: contraction 1..kmax, exponents log-uniform in
    [0.05, 1e4], normalised, centres uniform in a `box` A cube) and `nq` shell
    quartets whose canonical class is uniform over the 21 classes ss|ss ..
    dd|dd.  Returns (shell table, int32 (nq, 4) quartets)."""
    table = random_quartet_shells(nshell, seed=seed, kmax=kmax, box=box)
    rng = np.random.default_rng(seed + 1)
    ls = table["l"]
    byl = [np.where(ls == l)[0] for l in range(3)]
    cls = rng.integers(0, len(QUARTET_CLASSES), nq)
    q = np.empty((nq, 4), dtype=np.int32)
    for k, ((la, lb), (lc, ld)) in enumerate(QUARTET_CLASSES):
        sel = np.where(cls == k)[0]
        for col, l in enumerate((la, lb, lc, ld)):
            q[sel, col] = rng.choice(byl[l], len(sel))
    return table, q
