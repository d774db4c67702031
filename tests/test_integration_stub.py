"""The reference-side binding shown in INTEGRATION.md (``handle_from_molecule``
and ``jk``, the stub a maintainer adds to src/hf), executed as written.

Its input is the reference's own Molecule structure: ``mol.atoms[i].cgfs``,
each a ContractedGaussianFunction with ``shell``, ``expns``, ``coefs``
(shared by the components of a basis-file line), ``normalize_factors`` and
``center`` (src/hf/molecule.py:128-226).  The stand-in here is rebuilt from
the reference's own CGF data for water / STO-3G (tests/golden/h2o_sto3g.json,
written by the reference's molecule.py), grouped into atoms by centre.

* CPU: the shell descriptors the stub hands to sf_create (captured by a fake
  library object) equal the package's own shell table of the same molecule.
* GPU: the stub's handle and J/K, through the real library, equal
  FockBuilder.jk on the package's Molecule.
"""
import ctypes as C
import os
import re
import types

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
LIB_IN_DOC = 'C.CDLL("/path/to/segfault_py_gb300/csrc/libsegfock.so")'


def stub_source():
    text = open(os.path.join(REPO, "INTEGRATION.md")).read()
    blocks = re.findall(r"```python\n(.*?)```", text, flags=re.S)
    src = [b for b in blocks if "def handle_from_molecule" in b]
    assert len(src) == 1
    assert LIB_IN_DOC in src[0]
    return src[0]


def load_stub(lib_expr: str, extra: dict):
    """Run the stub with its library expression replaced by lib_expr."""
    ns = dict(extra)
    exec(compile(stub_source().replace(LIB_IN_DOC, lib_expr), "INTEGRATION.md", "exec"), ns)
    return ns


def reference_like_molecule(golden):
    """mol.atoms[i].cgfs from the reference's CGF records, atoms in order of first appearance."""
    atoms, centres = [], []
    for rec in golden["cgfs"]:
        g = types.SimpleNamespace(shell=list(rec["shell"]), expns=list(rec["expns"]), coefs=list(rec["coefs"]),
                                  normalize_factors=np.asarray(rec["nf"]), center=np.asarray(rec["center"]))
        for i, c in enumerate(centres):
            if np.allclose(c, g.center, atol=0, rtol=0):
                atoms[i].cgfs.append(g)
                break
        else:
            centres.append(g.center)
            atoms.append(types.SimpleNamespace(cgfs=[g]))
    return types.SimpleNamespace(atoms=atoms)


class _FakeFn:
    def __init__(self, name, owner):
        self.name, self.owner, self.argtypes, self.restype = name, owner, None, None

    def __call__(self, *args):
        if self.name == "sf_create":
            # copy the descriptors now: the stub frees its arrays on return
            # (the real library copies them inside the call)
            descs = C.cast(args[0], C.POINTER(self.owner.ns["ShellDesc"]))
            args = ([(d.l, d.nprim, d.atom, d.ao_offset, list(d.center), [d.exps[k] for k in range(d.nprim)],
                      [d.coefs[k] for k in range(d.nprim)]) for d in descs[:args[1]]],)
        self.owner.calls.append((self.name, args))
        return 0


class _FakeLib:
    def __init__(self):
        self.calls = []
        self.ns = None

    def __getattr__(self, name):
        f = _FakeFn(name, self)
        setattr(self, name, f)
        return f


def test_stub_shell_descs_match_package_shell_table(h2o_golden):
    from segfault_py_gb300.molecule import Molecule
    fake = _FakeLib()
    ns = load_stub("_FAKE", {"_FAKE": fake})
    fake.ns = ns
    ref_mol = reference_like_molecule(h2o_golden)
    ns["handle_from_molecule"](ref_mol)
    create = [a for n, a in fake.calls if n == "sf_create"]
    assert len(create) == 1
    descs = create[0][0]
    assert [n for n, _ in fake.calls] == ["sf_create", "sf_schwarz"]
    geo = h2o_golden["geometry_angstrom"]
    mol = Molecule.from_geometry([g[0] for g in geo], [g[1:] for g in geo], h2o_golden["basis"])
    t = mol.shell_table()
    assert len(descs) == len(t["l"])
    for s, (l, nprim, atom, ao, cen, e, c) in enumerate(descs):
        assert (l, nprim, atom, ao) == (t["l"][s], t["nprim"][s], t["atom"][s], t["ao_offset"][s])
        assert np.allclose(cen, t["center"][s], rtol=1e-15, atol=1e-15)
        o = t["prim_offset"][s]
        assert np.array_equal(np.array(e), t["exps"][o:o + nprim])
        assert np.allclose(np.array(c), t["coefs"][o:o + nprim], rtol=1e-14, atol=0)


@pytest.mark.gpu
def test_stub_jk_matches_fockbuilder(cuda, h2o_golden):
    import torch
    from segfault_py_gb300 import _lib
    from segfault_py_gb300.fock import FockBuilder
    from segfault_py_gb300.molecule import Molecule
    path = os.path.join(REPO, "segfault_py_gb300", "csrc", "libsegfock.so")
    _lib.lib()   # builds nothing; fails loudly if the library is missing
    ns = load_stub("C.CDLL(%r)" % path, {})
    ref_mol = reference_like_molecule(h2o_golden)
    h = ns["handle_from_molecule"](ref_mol)
    n = sum(len(a.cgfs) for a in ref_mol.atoms)
    P = np.asarray(h2o_golden["density"], dtype=np.float64)
    J, K = ns["jk"](h, P)
    geo = h2o_golden["geometry_angstrom"]
    mol = Molecule.from_geometry([g[0] for g in geo], [g[1:] for g in geo], h2o_golden["basis"])
    fb = FockBuilder(mol, device=cuda, cutoff=1e-12)
    Jr, Kr = fb.jk(torch.tensor(P, device=cuda), precision="fp64")
    assert J.shape == (n, n)
    scale = max(float(Jr.abs().max()), float(Kr.abs().max()))
    assert np.abs(J - Jr.cpu().numpy()).max() <= 1e-13 * scale
    assert np.abs(K - Kr.cpu().numpy()).max() <= 1e-13 * scale
    ns["lib"].sf_destroy(h)
    fb.close()
