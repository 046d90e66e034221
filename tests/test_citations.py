"""Every `file.f90:a-b` citation of the reference in this repository points at
real lines of the reference, and at the routine it names.

The reference checkout is found through the environment variable
RC_REFERENCE_DIR (its top directory, holding src/ and
inv-nozzle-no-BL-rocket/); without it the test is skipped.  For each citation
in the sources, headers, tests and notes:
- every cited line lies inside the cited file;
- where the same source line names a subroutine, function or module that the
  cited file defines, the cited range overlaps one of the named ones.
A few key citations are also checked to point at the definitions themselves.
"""
import os
import re

import pytest

from conftest import ROOT

REF = os.environ.get("RC_REFERENCE_DIR")
pytestmark = pytest.mark.skipif(not REF or not os.path.isdir(os.path.join(REF or "", "src")),
                                reason="RC_REFERENCE_DIR does not name a reference checkout")

CITE = re.compile(r"((?:[\w\-]+/)*)([\w\-]+\.f90):(\d+(?:-\d+)?(?:,\s?\d+(?:-\d+)?)*)")
# names too common in prose to tie a citation to a routine
GENERIC = {"main", "fun", "funx", "funy", "line", "face", "change", "contain", "relu", "swish", "softmax"}
SKIP_FILES = {"SURVEY.md", "VERDICT.md", "ADVICE.md", "BASELINE.md"}


def reference_files():
    out = {}
    for dp, _, fn in os.walk(REF):
        for f in fn:
            if f.endswith(".f90"):
                p = os.path.relpath(os.path.join(dp, f), REF)
                out.setdefault(f, []).append(p)
    return out


def routines(path):
    """(name, first line, last line) of every subroutine/function/module/program."""
    lines = open(os.path.join(REF, path), errors="replace").read().split("\n")
    stack, out = [], []
    for i, l in enumerate(lines, 1):
        s = l.strip().lower()
        if s.startswith("!"):
            continue
        m = re.match(r"^(?:recursive\s+|pure\s+|elemental\s+)*(?:(?:double precision|real|integer|logical)\s+)?"
                     r"(subroutine|function|module|program)\s+(\w+)", s)
        if m and not re.match(r"module\s+procedure", s):
            stack.append((m.group(2), i))
        e = re.match(r"^end\s*(subroutine|function|module|program)\b", s)
        if e and stack:
            n, a = stack.pop()
            out.append((n, a, i))
    return lines, out


def resolve(files, prefix, base):
    cands = files.get(base, [])
    if prefix:
        m = [c for c in cands if c.endswith(prefix + base)]
        if m:
            return m[0]
    src = [c for c in cands if c.startswith("src/")]
    return src[0] if len(src) == 1 else (cands[0] if cands else None)


def citations():
    for dp, dn, fn in os.walk(ROOT):
        dn[:] = [d for d in dn if d not in (".git", "_work", "gpurun_out", "_build", "__pycache__", "baseline")]
        for f in fn:
            if f in SKIP_FILES or not f.endswith((".py", ".cu", ".cuh", ".h", ".cpp", ".c", ".md")):
                continue
            p = os.path.join(dp, f)
            for ln, line in enumerate(open(p, errors="replace"), 1):
                for m in CITE.finditer(line):
                    yield os.path.relpath(p, ROOT), ln, line, m


def ranges(text):
    for part in text.split(","):
        a, _, b = part.strip().partition("-")
        yield int(a), int(b) if b else int(a)


def test_every_citation_points_inside_its_file_and_routine():
    files = reference_files()
    cache = {}
    bad = []
    n = 0
    for rel, ln, line, m in citations():
        n += 1
        path = resolve(files, m.group(1), m.group(2))
        if path is None:
            bad.append(f"{rel}:{ln}: {m.group(0)}: no such reference file")
            continue
        if path not in cache:
            cache[path] = routines(path)
        lines, rts = cache[path]
        nlines = len(lines) - (1 if lines and lines[-1] == "" else 0)
        rs = list(ranges(m.group(3)))
        for a, b in rs:
            if not (1 <= a <= b <= nlines):
                bad.append(f"{rel}:{ln}: {m.group(0)}: lines {a}-{b} outside 1-{nlines}")
        low = line.lower()
        named = [(nm, s, e) for nm, s, e in rts
                 if nm not in GENERIC and re.search(r"(?<![\w/])" + re.escape(nm) + r"(?!\w|\.f90)", low)]
        if named and not any(s <= b and a <= e for a, b in rs for _, s, e in named):
            bad.append(f"{rel}:{ln}: {m.group(0)} misses {[f'{nm}:{s}-{e}' for nm, s, e in named]}")
    assert n > 200
    assert not bad, "\n".join(bad)


@pytest.mark.parametrize("cite,name", [
    ("src/combustion_modeling/oxidizer.f90:53", "oxidizer_inlet_bc"),
    ("src/combustion_modeling/fuel.f90:54", "fuel_inlet_bc"),
    ("src/combustion_modeling/thermo_property.f90:78", "computegasparameter"),
    ("src/combustion_modeling/thermo_property.f90:114", "compute_enthalpy"),
    ("src/combustion_modeling/thermo_property.f90:146", "newton_temperature"),
    ("src/Time_LUSGS_steady.f90:4", "lu_sgs_stage"),
    ("src/Time_LUSGS_steady.f90:32", "lu_sgs_steady"),
    ("src/update_flow_variables.f90:4", "update_primitve_variables"),
    ("src/update_flow_variables.f90:90", "update_ghostcell_variables"),
    ("src/la_math.f90:120", "advanced_linear_solve_lapack"),
])
def test_key_definitions(cite, name):
    """The routines the hot path restates start where the code cites them."""
    path, ln = cite.rsplit(":", 1)
    lines = open(os.path.join(REF, path), errors="replace").read().split("\n")
    assert re.match(r"\s*(subroutine|function)\s+" + name + r"\b", lines[int(ln) - 1], re.I), lines[int(ln) - 1]
    found = any(f"{os.path.basename(path)}:{ln}" in line for _, _, line, _ in citations())
    assert found, f"no citation of {os.path.basename(path)}:{ln}"
