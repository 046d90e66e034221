"""Fixture: the reference's own combustor mesh, inv-nozzle-no-BL-rocket/rocket2.msh.

Reads the gmsh 4.1 file of a reference checkout (path from the environment
variable RC_REFERENCE_DIR, or the first argument) with
rocketcombustor_gb300.gmsh.read_msh, the restatement of readgmsh.f90 for one
partition, and stores what a case needs in tests/golden/rocket2_mesh.npz:
node coordinates (NNT, 2) float64, triangles (NE, 3) int32 as 1-based node ids
in file order, and the boundary edges with their solver codes (the physical
tags mapped by readgmsh.f90:68-73).  The tests rebuild the mesh from it
(`load_mesh`), so the reference checkout is not needed to run them.
"""
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
OUT = os.path.join(HERE, "rocket2_mesh.npz")


def load_mesh():
    """The fixture as a rocketcombustor_gb300.cases.Mesh."""
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from rocketcombustor_gb300.cases import Mesh

    with np.load(OUT) as z:
        codes, starts = z["bnd_code"], z["bnd_start"]
        pairs = z["bnd_pairs"].astype(np.int64)
        bnd = [(int(codes[k]), pairs[starts[k]:starts[k + 1]]) for k in range(codes.size)]
        return Mesh(coor=z["coor"].copy(), cells=z["cells"].astype(np.int64), boundaries=bnd, nx=0, ny=0)


def main(path=None):
    if ROOT not in sys.path:
        sys.path.insert(0, ROOT)
    from rocketcombustor_gb300 import gmsh

    path = path or os.path.join(os.environ["RC_REFERENCE_DIR"], "inv-nozzle-no-BL-rocket", "rocket2.msh")
    m = gmsh.read_msh(path)
    codes = np.array([c for c, _ in m.boundaries], dtype=np.int32)
    starts = np.cumsum([0] + [len(p) for _, p in m.boundaries]).astype(np.int64)
    pairs = np.concatenate([p for _, p in m.boundaries]).astype(np.int32)
    np.savez_compressed(OUT, coor=m.coor, cells=m.cells.astype(np.int32), bnd_code=codes, bnd_start=starts,
                        bnd_pairs=pairs)
    print(OUT, m.cells.shape, m.coor.shape, {int(c): len(p) for c, p in m.boundaries})


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else None)
