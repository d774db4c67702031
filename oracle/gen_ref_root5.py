"""Recipe: build the reference's own Rys root fits into oracle/_ref/ (oracle only).

The reference engine (src/hf/core/core.f90) is Fortran and needs GSL; neither a
Fortran compiler nor GSL is available, so the f2py module cannot be built
(core.f90:1).  Its Rys root routine ``root5`` (core.f90:232-812) is, however,
straight-line arithmetic.  This script reads that subroutine from the reference
source where it lies and transcribes it mechanically into C (continuation lines
joined, D exponents -> e, IF/ELSE IF/ELSE/END IF -> braces, SQRT/EXP -> libm),
then compiles it into ``oracle/_ref/librefroot5.so`` exporting
``ref_root5(const double *x, double *res10)`` with the Fortran calling
convention of ``root5(x, res)``: res[0:5] = t^2 = RT/(1+RT), res[5:10] weights.

Outputs go only to oracle/_ref/ (git-ignored).  Nothing generated is committed.
The oracle uses the library to pin its own root generator and, when present,
as the root provider of the timed CPU baseline (the reference's arithmetic).

Usage: python oracle/gen_ref_root5.py [path/to/core.f90]
(default: $SEGFAULT_PY_REFERENCE/src/hf/core/core.f90).  Where the reference
source is absent but oracle/_ref/ref_root5.c was transcribed earlier (and
copied along with the working tree), only the compile step runs.
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# the reference checkout this recipe reads: $SEGFAULT_PY_REFERENCE, else its usual place here
DEFAULT_SRC = os.path.join(os.environ.get("SEGFAULT_PY_REFERENCE", "/root/reference"), "src/hf/core/core.f90")


def extract_root5(lines):
    start = end = None
    for i, l in enumerate(lines):
        s = l.strip().lower()
        if s.startswith("subroutine root5"):
            start = i
        elif start is not None and s.startswith("end subroutine"):
            end = i
            break
    if start is None or end is None:
        raise RuntimeError("subroutine root5 not found")
    return lines[start + 1:end]


def join_continuations(lines):
    out, buf = [], ""
    for l in lines:
        s = l.split("!")[0].rstrip()
        if s.endswith("&"):
            buf += s[:-1] + " "
            continue
        buf += s
        if buf.strip():
            out.append(buf.strip())
        buf = ""
    return out


def cexpr(s):
    s = re.sub(r"(\d)[dD]([+-]?\d+)", r"\1e\2", s)
    s = re.sub(r"(\d\.?\d*)_8\b", r"\1", s)
    s = re.sub(r"\b([A-Za-z]\w*)\*\*3\b", r"(\1*\1*\1)", s)
    s = re.sub(r"\b([A-Za-z]\w*)\*\*2\b", r"(\1*\1)", s)
    s = s.replace(".LT.", "<").replace(".lt.", "<")
    s = re.sub(r"\bSQRT\s*\(", "sqrt(", s, flags=re.I)
    s = re.sub(r"\bEXP\s*\(", "exp(", s, flags=re.I)
    s = re.sub(r"\bx\b", "X", s)
    return s


def transcribe(body):
    stmts = join_continuations(body)
    params, code, ind = [], [], 1
    for st in stmts:
        low = st.lower()
        if low.startswith("double precision"):
            if "parameter" in low:
                name, val = st.split("::")[1].split("=")
                params.append("    const double %s = %s;" % (name.strip(), cexpr(val.strip())))
            continue
        m = re.match(r"^(ELSE\s+)?IF\s*\((.*)\)\s*THEN$", st, flags=re.I)
        if m:
            cond = cexpr(m.group(2).strip())
            if m.group(1):
                code.append("    " * (ind - 1) + "} else if (%s) {" % cond)
            else:
                code.append("    " * ind + "if (%s) {" % cond)
                ind += 1
            continue
        if re.match(r"^ELSE$", st, flags=re.I):
            code.append("    " * (ind - 1) + "} else {")
            continue
        if re.match(r"^END\s*IF$", st, flags=re.I):
            ind -= 1
            code.append("    " * ind + "}")
            continue
        m = re.match(r"^res\s*=\s*\(/(.*)/\)$", st, flags=re.I)
        if m:
            items = [cexpr(t.strip()) for t in m.group(1).split(",")]
            for k, it in enumerate(items):
                code.append("    res[%d] = %s;" % (k, it))
            continue
        m = re.match(r"^([A-Za-z]\w*)\s*=\s*(.*)$", st)
        if m:
            code.append("    " * ind + "%s = %s;" % (m.group(1), cexpr(m.group(2))))
            continue
        raise RuntimeError("untranscribed statement: %r" % st)
    head = ["/* Generated by oracle/gen_ref_root5.py from core.f90 subroutine root5.",
            " * Not part of the repository history (oracle/_ref/ is git-ignored). */",
            "#include <math.h>",
            "void ref_root5(const double *xp, double *res)",
            "{",
            "    const double X = *xp;"]
    decl = ["    double RT1 = 0, RT2 = 0, RT3 = 0, RT4 = 0, RT5 = 0;",
            "    double WW1 = 0, WW2 = 0, WW3 = 0, WW4 = 0, WW5 = 0, E = 0, Y = 0, XXX = 0;",
            "    (void)E; (void)Y; (void)XXX;"]
    return "\n".join(head + params + decl + code + ["}"]) + "\n"


def compile_c(cpath):
    so = os.path.join(OUT, "librefroot5.so")
    subprocess.check_call(["gcc", "-O2", "-shared", "-fPIC", "-o", so, cpath, "-lm"])
    print("built", so)
    return so


def main(src=None):
    src = src or DEFAULT_SRC
    cpath = os.path.join(OUT, "ref_root5.c")
    if not os.path.exists(src):
        # a machine without the reference checkout: the transcription made
        # where the source was (git-ignored, copied along with the working
        # tree) is compiled for this machine's architecture
        if os.path.exists(cpath):
            compile_c(cpath)
            return 0
        print("reference source not found: %s (oracle/_ref not built)" % src)
        return 1
    os.makedirs(OUT, exist_ok=True)
    with open(src) as f:
        body = extract_root5(f.read().split("\n"))
    c = transcribe(body)
    with open(cpath, "w") as f:
        f.write(c)
    compile_c(cpath)
    return 0


if __name__ == "__main__":
    sys.exit(main(sys.argv[1] if len(sys.argv) > 1 else None))
