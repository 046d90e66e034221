"""Generate the golden vectors under tests/golden/.

The reference (Fortran 90 with MPI and LAPACK) cannot be built on either
machine and ships no tests, logs or outputs, so these vectors come from the
CPU FP64 oracle (oracle/rc_oracle.cpp), which restates the reference line by
line.  They fix both sides of the parity tests to committed numbers:
  * the case inputs are committed as the reference's own file formats
    (grid1.in, fvp1.sav, flow/ and combustion/ .in files), so the vectors do
    not depend on the case generator or on the host's libm;
  * the outputs are the oracle's state after a fixed number of iterations.

Cases (all 24 x 6 cells along x/y, 288 triangles):
  t1   inviscid perfect gas (NVar 4), 50 steady LU-SGS iterations
       (lu_sgs_stage, src/Time_LUSGS_steady.f90:4-30);
  t2   reacting viscous, 4 species (NVar 7), 50 steady iterations;
  t2u  t2 under the shipped dual-time BDF2 scheme (src/Time_BDF2.f90:4-69,
       driver src/fvm2d.f90:80-99), 3 physical steps.

Each <case>.npz holds PA, WA and hWA (the oracle's arrays, [cell, var]),
the per-iteration residual norms Res(1:NVar), romax of the steady cases
(src/residual.f90:4-20), the inner iteration counts of the unsteady case,
and `digest`, the SHA-256 of the case directory's files.

Run from the repository root:  python tests/golden/make_golden.py
(--outputs-only keeps the committed case directories and recomputes the
vectors from them.)
"""
from __future__ import annotations

import argparse
import hashlib
import os
import shutil
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

# case -> (kind, iterations or physical steps)
CASES = {"t1": ("steady", 50), "t2": ("steady", 50), "t2u": ("unsteady", 3)}


def case_dir(name: str) -> str:
    return os.path.join(HERE, name)


def digest(d: str) -> str:
    """SHA-256 over the relative paths and bytes of every file of a case."""
    h = hashlib.sha256()
    for root, dirs, files in os.walk(d):
        dirs.sort()
        for f in sorted(files):
            p = os.path.join(root, f)
            h.update(os.path.relpath(p, d).replace(os.sep, "/").encode())
            with open(p, "rb") as fh:
                h.update(fh.read())
    return h.hexdigest()


def working_copy(name: str, into: str) -> str:
    """Copy of the committed case (the solvers may write next to their inputs)."""
    dst = os.path.join(into, name)
    shutil.copytree(case_dir(name), dst)
    return dst


def load(name: str) -> dict:
    with np.load(os.path.join(HERE, name + ".npz")) as z:
        return {k: z[k] for k in z.files}


def oracle_outputs(name: str, d: str) -> dict:
    import oracle

    kind, n = CASES[name]
    o = oracle.Oracle(d)
    out = {}
    if kind == "steady":
        out["history"] = o.run(n, history=True)
    else:
        out["inner"] = np.array([o.unsteady_step(i)[0] for i in range(1, n + 1)], dtype=np.int32)
    for a in ("PA", "WA", "hWA"):
        out[a] = o.array(a).copy()
    o.close()
    return out


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--outputs-only", action="store_true")
    args = ap.parse_args()
    from rocketcombustor_gb300 import cases

    for name in CASES:
        if not args.outputs_only:
            if os.path.isdir(case_dir(name)):
                shutil.rmtree(case_dir(name))
            cases.make_case(case_dir(name), name)
        with tempfile.TemporaryDirectory() as tmp:
            out = oracle_outputs(name, working_copy(name, tmp))
        np.savez_compressed(os.path.join(HERE, name + ".npz"), digest=np.array(digest(case_dir(name))), **out)
        print(name, {k: v.shape for k, v in out.items()})


if __name__ == "__main__":
    main()
