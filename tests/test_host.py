"""Host-side logic (no GPU): basis ingestion parity, shell tables, geometry
generators, the C ABI exports and the library's Rys root tables."""
import re

import numpy as np
import pytest

from conftest import REPO, load_golden
from oracle import oracle as O
from segfault_py_gb300 import geometry as G
from segfault_py_gb300.molecule import Molecule


def test_molecule_matches_reference_cgfs(h2o_golden):
    mol = Molecule.from_geometry(["O", "H", "H"], [[0, 0, 0], [0.757, 0.587, 0], [-0.757, 0.587, 0]], "sto-3g")
    assert abs(mol.e_nuc - h2o_golden["e_nuc"]) < 1e-13
    assert len(mol.cgfs) == len(h2o_golden["cgfs"]) == 7
    for mine, ref in zip(mol.cgfs, h2o_golden["cgfs"]):
        assert list(mine.shell) == ref["shell"]
        np.testing.assert_allclose(mine.coefs, ref["coefs"], rtol=1e-15)
        np.testing.assert_allclose(mine.normalize_factors, ref["nf"], rtol=1e-15)
        np.testing.assert_allclose(mine.center, ref["center"], rtol=1e-15)


def test_shell_table_reproduces_component_coefficients():
    s, x = G.water_cluster(2, seed=3)
    mol = Molecule.from_geometry(s, x, "6-31g*")
    t = mol.shell_table()
    from segfault_py_gb300.fock import _comp_factor
    for sh in mol.shells:
        for cg in sh.cgfs:
            eff = np.asarray(cg.coefs) * cg.normalize_factors
            np.testing.assert_allclose(sh.coefs * _comp_factor(cg.shell), eff, rtol=1e-14)
    assert t["ao_offset"][-1] + (t["l"][-1] + 1) * (t["l"][-1] + 2) // 2 == mol.nao == 38


def test_config_sizes():
    for n, nao, nsh in [(8, 152, 80), (16, 304, 160)]:
        s, x = G.water_cluster(n)
        m = Molecule.from_geometry(s, x, "6-31g*")
        assert (m.nao, len(m.shells)) == (nao, nsh)
    s, x = G.alkane(20)
    m = Molecule.from_geometry(s, x, "6-31g**")
    assert (m.nao, len(m.shells), m.natom) == (510, 246, 62)


def test_water_cluster_is_seeded():
    a = G.water_cluster(8, seed=0)[1]
    b = G.water_cluster(8, seed=0)[1]
    c = G.water_cluster(8, seed=1)[1]
    assert np.array_equal(a, b) and not np.array_equal(a, c)
    # monomer geometry preserved by the rotation
    for k in range(8):
        o, h1, h2 = a[3 * k: 3 * k + 3]
        assert abs(np.linalg.norm(h1 - o) - np.hypot(0.757, 0.587)) < 1e-12
        assert abs(np.linalg.norm(h2 - o) - np.hypot(0.757, 0.587)) < 1e-12


def test_basis_not_available():
    from segfault_py_gb300.molecule import BasisSetNotAvailableError
    with pytest.raises(BasisSetNotAvailableError):
        Molecule.from_geometry(["N"], [[0, 0, 0]], "sto-3g")


def _header_symbols():
    txt = open(f"{REPO}/include/segfock.h").read()
    return sorted(set(re.findall(r"\b(sf_[a-z_0-9]+)\s*\(", txt)))


def test_library_exports_every_declared_symbol():
    from segfault_py_gb300 import _lib
    L = _lib.lib()
    syms = _header_symbols()
    assert len(syms) >= 12
    for s in syms:
        assert hasattr(L, s), s


def test_create_rejects_bad_shells_without_gpu():
    import ctypes as C
    from segfault_py_gb300 import _lib
    L = _lib.lib()
    e = np.array([1.0]); c = np.array([1.0])
    arr = (_lib.ShellDesc * 1)()
    arr[0].l = 3
    arr[0].nprim = 1
    arr[0].ao_offset = 0
    arr[0].exps = e.ctypes.data_as(C.POINTER(C.c_double))
    arr[0].coefs = c.ctypes.data_as(C.POINTER(C.c_double))
    h = C.c_void_p()
    assert L.sf_create(C.cast(arr, C.c_void_p), 1, C.byref(h)) == -2
    assert b"l > 2" in L.sf_last_error()
    arr[0].l = 0
    e[0] = -1.0
    assert L.sf_create(C.cast(arr, C.c_void_p), 1, C.byref(h)) == -1
    assert L.sf_create(None, 0, C.byref(h)) == -1


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5])
def test_library_root_tables_vs_oracle_exact(n):
    from segfault_py_gb300 import _lib
    L = _lib.lib()
    u = np.zeros(n); w = np.zeros(n)
    xs = np.concatenate([[0.0, 1e-12, 0.5, 63.999, 64.0, 64.001, 99.0, 1e3, 1e6], np.linspace(0.01, 70, 157)])
    for x in xs:
        ue, we = O.rys_roots_exact(n, x)
        assert L.sf_rys_roots_host(n, float(x), 0, u.ctypes.data, w.ctypes.data) == 0
        np.testing.assert_allclose(u, ue, rtol=5e-14)
        np.testing.assert_allclose(w, we, rtol=5e-14)
        assert L.sf_rys_roots_host(n, float(x), 1, u.ctypes.data, w.ctypes.data) == 0
        np.testing.assert_allclose(u, ue, rtol=3e-6)
        np.testing.assert_allclose(w, we, rtol=3e-6)


def test_library_roots_vs_reference_root5():
    from segfault_py_gb300 import _lib
    L = _lib.lib()
    g = load_golden("root5_ref.json")
    u = np.zeros(5); w = np.zeros(5)
    for x, res in zip(g["x"], g["res"]):
        L.sf_rys_roots_host(5, float(x), 0, u.ctypes.data, w.ctypes.data)
        np.testing.assert_allclose(np.concatenate([u, w]), res, rtol=2e-12)


def test_nuclear_repulsion_gradient_fd():
    from segfault_py_gb300.grad import nuclear_repulsion_gradient
    from segfault_py_gb300.molecule import BOHR
    s, x = G.water_cluster(2, seed=9)
    m = Molecule.from_geometry(s, x, "sto-3g")
    g = nuclear_repulsion_gradient(m)
    h = 1e-5
    for a in range(m.natom):
        for d in range(3):
            xp, xm = x.copy(), x.copy()
            xp[a, d] += h * BOHR
            xm[a, d] -= h * BOHR
            fd = (Molecule.from_geometry(s, xp, "sto-3g").e_nuc - Molecule.from_geometry(s, xm, "sto-3g").e_nuc) / (2 * h)
            assert abs(fd - g[a, d]) < 1e-7


def test_ctypes_structs_match_header_layout(tmp_path):
    """Every struct of include/segfock.h that the binding mirrors has the
    same size and field offsets in C (gcc on the header) and in ctypes."""
    import ctypes as C
    import shutil
    import subprocess
    from segfault_py_gb300 import _lib
    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    mirrors = {"sf_shell_desc": _lib.ShellDesc, "sf_stats": _lib.Stats, "sf_slice_info": _lib.SliceInfo,
               "sf_tune_entry": _lib.TuneEntry}
    lines = ["#include <stddef.h>", "#include <stdio.h>", '#include "segfock.h"', "int main(void) {"]
    for cname, py in mirrors.items():
        lines.append('  printf("%s size %%zu\\n", sizeof(%s));' % (cname, cname))
        for f, _ in py._fields_:
            lines.append('  printf("%s %s %%zu\\n", offsetof(%s, %s));' % (cname, f, cname, f))
    lines += ["  return 0;", "}"]
    src = tmp_path / "layout.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "layout"
    subprocess.run([cc, "-std=c11", "-I", f"{REPO}/include", str(src), "-o", str(exe)], check=True)
    out = subprocess.run([str(exe)], check=True, capture_output=True, text=True).stdout.split("\n")
    got = {tuple(l.split()[:2]): int(l.split()[2]) for l in out if l.strip()}
    for cname, py in mirrors.items():
        assert got[(cname, "size")] == C.sizeof(py), cname
        for f, _ in py._fields_:
            assert got[(cname, f)] == getattr(py, f).offset, (cname, f)


def test_timeline_table_bins_and_tiers():
    from segfault_py_gb300.profile_build import timeline_table

    class FakeBuilder:
        def slice_info(self):
            base = {"la": 0, "lb": 0, "lc": 0, "ld": 0, "threads_per_quartet": 1, "quartets": 10}
            return [dict(base, start_ms=0.0, ms=0.1, precision=1, stream=0),
                    dict(base, start_ms=0.05, ms=0.1, precision=2, stream=1),
                    dict(base, start_ms=0.15, ms=0.05, precision=1, stream=0)]

    rows = timeline_table(FakeBuilder(), bin_ms=0.05)
    assert rows[0].startswith("build span 0.2000 ms, launch time summed 0.2500 ms")
    assert "f32: 2 launches, first start 0.0000 ms, last end 0.2000 ms, summed 0.1500 ms" in rows[1]
    assert "dd: 1 launches, first start 0.0500 ms, last end 0.1500 ms, summed 0.1000 ms" in rows[2]
    # bins [0,.05) [.05,.1) [.1,.15) [.15,.2) [.2,.25): 1, 2, 1, 1, 0 launches in flight
    assert rows[3].endswith("1.0 2.0 1.0 1.0 0.0")
    assert [r.split()[0] for r in rows[4:]] == ["start=", "start=", "start="]


def test_bench_dominant_kernel_sums_launches_of_one_kernel():
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", f"{REPO}/bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)

    def sl(cls, prec, ms, flop=1.0):
        return {"la": cls[0], "lb": cls[1], "lc": cls[2], "ld": cls[3], "precision": prec, "ms": ms,
                "flop_alg": flop, "threads_per_quartet": 1}

    slices = [sl((2, 0, 1, 1), 2, 0.05), sl((1, 0, 0, 0), 1, 0.03), sl((1, 0, 0, 0), 1, 0.04),
              sl((1, 0, 0, 0), 2, 0.02)]
    top, group, name = bench.dominant_kernel(slices)
    assert name == "jk_kernel<1,0,0,0,fp32>"
    assert len(group) == 2 and top["ms"] == 0.04


def test_bench_traffic_table_is_keyed_to_the_kernel_sources(tmp_path):
    """The committed ncu traffic table is used only for the kernel sources it
    was measured on: a table with another source hash gives traffic = null."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("bench_mod", f"{REPO}/bench.py")
    bench = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(bench)
    t = tmp_path / "traffic.txt"
    t.write_text("# csrc_sha16 %s\njk_kernel<1,0,0,0,fp32> 1234\n" % bench.csrc_hash())
    bench.TRAFFIC_TABLE = str(t)
    v, src = bench.ncu_traffic("jk_kernel<1,0,0,0,fp32>")
    assert v == 1234.0 and "ncu capture" in src
    assert bench.ncu_traffic("jk_kernel<2,0,0,0,dd>")[0] is None
    t.write_text("# csrc_sha16 0000000000000000\njk_kernel<1,0,0,0,fp32> 1234\n")
    v, src = bench.ncu_traffic("jk_kernel<1,0,0,0,fp32>")
    assert v is None and "stale" in src


def test_profile_traffic_table_from_ncu_csv(tmp_path):
    """The DRAM table builder: ncu launch rows mapped to kernel families,
    bytes summed per family and divided by the families' quartets."""
    from segfault_py_gb300 import profile_traffic as PT
    assert PT.family_of_ncu("void sf::jk_kernel<(int)1, (int)0, (int)0, (int)0, float, (int)1>(sf::KParams)") \
        == "jk_kernel<1,0,0,0,fp32>"
    assert PT.family_of_ncu("void sf::jk_kernel<2, 1, 1, 0, sf::dd, 4>(sf::KParams)") == "jk_kernel<2,1,1,0,dd>"
    assert PT.family_of_ncu("void sf::grad_kernel<2, 1, 1, 0, double, 8>(sf::KParams)") is None
    hdr = '"ID","Process ID","Process Name","Host Name","Kernel Name","Context","Stream","Block Size","Grid Size",' \
          '"Device","CC","Section Name","Metric Name","Metric Unit","Metric Value"\n'
    rows = []
    for lid, name, rd, wr in ((0, "void sf::jk_kernel<1, 0, 0, 0, float, 1>(x)", "2.5", "0.5"),
                              (1, "void sf::jk_kernel<1, 0, 0, 0, float, 1>(x)", "1,000", "0"),
                              (2, "void sf::jk_kernel<2, 2, 2, 2, double, 32>(x)", "0.5", "0.25")):
        unit = "byte" if lid == 1 else "Kbyte"
        for metric, val in (("dram__bytes_read.sum", rd), ("dram__bytes_write.sum", wr)):
            rows.append('"%d","1","p","h","%s","1","7","(128, 1, 1)","(9, 1, 1)","0","10.3","","%s","%s","%s"\n'
                        % (lid, name, metric, unit, val))
    (tmp_path / "dram.csv").write_text("==PROF== header line\n" + hdr + "".join(rows))
    (tmp_path / "slices.log").write_text(
        "(10|00) f32 T= 1 q=     1000 pq=   8000 ms=  0.1 share= 50.0% GF/s=  1.0\n"
        "(10|00) f32 T= 8 q=      500 pq=   4000 ms=  0.1 share= 25.0% GF/s=  1.0\n"
        "(22|22) f64 T=32 q=       25 pq=     25 ms=  0.1 share= 25.0% GF/s=  1.0\n")
    out = tmp_path / "table.txt"
    PT.main(["--csv", str(tmp_path / "dram.csv"), "--slices", str(tmp_path / "slices.log"), "--out", str(out)])
    table = {t.split()[0]: t.split() for t in out.read_text().splitlines() if not t.startswith("#")}
    assert abs(float(table["jk_kernel<1,0,0,0,fp32>"][1]) - (3000.0 + 1000.0) / 1500) < 1e-4   # written to 4 decimals
    assert table["jk_kernel<1,0,0,0,fp32>"][2:] == ["2", "1500"]
    assert abs(float(table["jk_kernel<2,2,2,2,fp64>"][1]) - 750.0 / 25) < 1e-4
    assert ("# csrc_sha16 " + PT.csrc_hash()) in out.read_text()


ROWS_CHECK = r'''
#include <cstdio>
#include "classes.h"
#include "quartet.cuh"
using namespace sf;

// lane t's k-th accumulator holds output (t + (k / INNER) T) INNER + k % INNER
// (the mapping of Grp::out, a device function)
template <int LA, int LB, int LC, int LD, typename R, int T>
static int check_class() {
  using Q = QC<LA, LB, LC, LD>;
  using GP = Grp<LA, LB, LC, LD, R, T>;
  int bad = 0;
  static int seen[1296];
  for (int o = 0; o < Q::NABCD; ++o) seen[o] = 0;
  for (int t = 0; t < T; ++t)
    for (int k = 0; k < GP::NPER; ++k) {
      const int o = (t + (k / GP::INNER) * T) * GP::INNER + k % GP::INNER;
      if (o < Q::NABCD) ++seen[o];
    }
  for (int o = 0; o < Q::NABCD; ++o) bad += seen[o] != 1;
  if (GP::ROWS * GP::INNER != Q::NABCD || GP::RPER * T < GP::ROWS) ++bad;
  if (GP::INNER > 1) {
    for (int row = 0; row < GP::ROWS; ++row)
      for (int e = 0; e < GP::INNER; ++e)
        for (int d = 0; d < 3; ++d)
          bad += Q::toff(row * GP::INNER + e, d) !=
                 Q::toff(row * GP::INNER, d) - cart_e(GP::LI, 0, d) + cart_e(GP::LI, e, d);
  }
  if (2 * Q::NR * Q::SZ + Q::SZ >= 1024) ++bad;
  printf("%d%d%d%d %s %d %d %d\n", LA, LB, LC, LD, sizeof(R) == 4 ? "fp32" : "fp64", GP::INNER, GP::NPER, bad);
  return bad;
}

int main() {
  int bad = 0;
#define SF_CHK(id, la, lb, lc, ld, t64, t32)                     \
  if (t32 > 1) bad += check_class<la, lb, lc, ld, float, t32>(); \
  if (t64 > 1) bad += check_class<la, lb, lc, ld, double, t64>();
  SF_CLASS_LIST(SF_CHK)
#undef SF_CHK
  return bad != 0;
}
'''


def test_group_rows_cover_outputs_and_reuse_table_factors(tmp_path):
    """The FP32 group kernels' row layout (quartet.cuh, Grp / eval_grp),
    checked on the host against the library's own table offsets for every
    class with more than one lane per quartet: the lanes' accumulators cover
    each output exactly once; a row's outputs read 2-D factors that differ
    only by the inner shell's exponent (consecutive entries); the packed
    10-bit offsets fit; FP64 groups keep one output per row."""
    import os
    import shutil
    import subprocess
    nvcc = shutil.which("nvcc")
    if nvcc is None and os.path.exists("/usr/local/cuda/bin/nvcc"):
        nvcc = "/usr/local/cuda/bin/nvcc"
    if nvcc is None:
        pytest.skip("no nvcc")
    src = tmp_path / "rows.cu"
    src.write_text(ROWS_CHECK)
    exe = tmp_path / "rows"
    csrc = f"{REPO}/segfault_py_gb300/csrc"
    subprocess.run([nvcc, "-std=c++17", "--expt-relaxed-constexpr", "-gencode", "arch=compute_103a,code=sm_103a",
                    "-I", f"{REPO}/include", "-I", csrc, str(src), "-o", str(exe)], check=True)
    r = subprocess.run([str(exe)], capture_output=True, text=True)
    rows = [l.split() for l in r.stdout.splitlines() if l.strip()]
    assert r.returncode == 0, r.stdout
    assert all(int(x[-1]) == 0 for x in rows)
    inner = {(x[0], x[1]): int(x[2]) for x in rows}
    assert inner[("2222", "fp32")] == 6 and inner[("2121", "fp32")] == 3 and inner[("2220", "fp32")] == 6
    assert all(v == 1 for (k, p), v in inner.items() if p == "fp64")
