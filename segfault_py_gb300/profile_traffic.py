"""DRAM traffic per quartet of the J/K class kernels, from one ncu capture.

    python -m segfault_py_gb300.profile_build --nwater 8 --precision mixed_df --slices --builds 1 > slices.log
    ncu --metrics dram__bytes_read.sum,dram__bytes_write.sum,gpu__time_duration.sum --clock-control none \\
        --kernel-name-base demangled -k regex:jk_kernel --csv --log-file dram.csv \\
        python -m segfault_py_gb300.profile_build --nwater 8 --precision mixed_df --slices --builds 1
    python -m segfault_py_gb300.profile_traffic --csv dram.csv --slices slices.log --out table.txt

The --slices build serialises its launches on one stream, so ncu's launch list
and the slice table list the same launches.  Per kernel family (class and
arithmetic: `jk_kernel<la,lb,lc,ld,fp64|fp32|dd>`) the table holds the DRAM
bytes (read + write) summed over its launches divided by the quartets those
launches processed, and the hash of the kernel sources it was measured on;
bench.py scales it by the quartets of the launch it reports and ignores a
table measured on other sources.
"""
from __future__ import annotations

import argparse
import collections
import csv
import hashlib
import os
import re

PKG = os.path.dirname(os.path.abspath(__file__))


def csrc_hash() -> str:
    """sha256 (first 16 hex digits) over the library's CUDA/C++ sources."""
    d = os.path.join(PKG, "csrc")
    h = hashlib.sha256()
    for f in sorted(os.listdir(d)):
        if f.endswith((".cu", ".cuh", ".h", ".cpp")):
            h.update(f.encode())
            with open(os.path.join(d, f), "rb") as fh:
                h.update(fh.read())
    return h.hexdigest()[:16]


_ARITH = {"double": "fp64", "float": "fp32", "sf::dd": "dd", "dd": "dd"}


def family_of_ncu(name: str):
    m = re.search(r"jk_kernel<\s*(?:\(int\))?(\d+),\s*(?:\(int\))?(\d+),\s*(?:\(int\))?(\d+),\s*(?:\(int\))?(\d+),"
                  r"\s*([\w:]+)", name)
    if not m:
        return None
    return "jk_kernel<%s,%s,%s,%s,%s>" % (m.group(1), m.group(2), m.group(3), m.group(4), _ARITH[m.group(5)])


def family_of_slice(line: str):
    m = re.match(r"\((\d)(\d)\|(\d)(\d)\) (f64|f32|dd)\s+T=\s*\d+ q=\s*(\d+)", line.strip())
    if not m:
        return None
    arith = {"f64": "fp64", "f32": "fp32", "dd": "dd"}[m.group(5)]
    return "jk_kernel<%s,%s,%s,%s,%s>" % (m.group(1), m.group(2), m.group(3), m.group(4), arith), int(m.group(6))


def read_ncu(path):
    """{family: [DRAM bytes per launch]} from an ncu --csv log."""
    rows = list(csv.reader(open(path)))
    hdr = next(i for i, r in enumerate(rows) if "Kernel Name" in r)
    h = rows[hdr]
    ki, mi, vi, ui, ii = (h.index(k) for k in ("Kernel Name", "Metric Name", "Metric Value", "Metric Unit", "ID"))
    scale = {"byte": 1.0, "Kbyte": 1e3, "Mbyte": 1e6, "Gbyte": 1e9}
    per = collections.defaultdict(float)
    names = {}
    for r in rows[hdr + 1:]:
        if len(r) <= vi or not r[mi].startswith("dram__bytes"):
            continue
        per[r[ii]] += float(r[vi].replace(",", "")) * scale.get(r[ui], 1.0)
        names[r[ii]] = r[ki]
    out = collections.defaultdict(list)
    for lid in sorted(per, key=int):
        fam = family_of_ncu(names[lid])
        if fam:
            out[fam].append(per[lid])
    return out


def main(argv=None):
    ap = argparse.ArgumentParser()
    ap.add_argument("--csv", required=True)
    ap.add_argument("--slices", required=True)
    ap.add_argument("--out", required=True)
    a = ap.parse_args(argv)
    bytes_of = read_ncu(a.csv)
    quartets = collections.defaultdict(int)
    for line in open(a.slices):
        r = family_of_slice(line)
        if r:
            quartets[r[0]] += r[1]
    with open(a.out, "w") as f:
        f.write("# DRAM bytes (read + write) per quartet of each J/K kernel family, one ncu capture of a serialised\n")
        f.write("# (H2O)8 6-31G* FP32 + double-float build (python -m segfault_py_gb300.profile_traffic, which lists the\n")
        f.write("# commands); columns: kernel, bytes per quartet, launches, quartets\n")
        f.write("# csrc_sha16 %s\n" % csrc_hash())
        for fam in sorted(bytes_of):
            q = quartets.get(fam, 0)
            if q > 0:
                f.write("%s %.4f %d %d\n" % (fam, sum(bytes_of[fam]) / q, len(bytes_of[fam]), q))


if __name__ == "__main__":
    main()
