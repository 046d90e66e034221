"""gmsh 4.1 ASCII meshes as RocketCombustor cases.

Restates the reference's mesh tooling for one partition:
- `readgmsh` (inv-nozzle-no-BL-rocket/readgmsh.f90:79-456) reads the
  $Entities, $Nodes and $Elements sections, keeps the 2-D elements as cells in
  file order and collects the boundary edges by the physical tag of their
  curve;
- the physical tags map to the solver's boundary codes by its system table
  (readgmsh.f90:68-73): 1 -> 4 (fuel inlet), 2 -> 3 (oxidizer inlet),
  3 -> 1 (no-slip wall), 4 -> 5 (outlet), 5 -> 2 (symmetry), 6 -> 6 (slip wall);
- the partition tool keeps the global cell order in a partition
  (src-meshpartition/MeshPre.f90:117-121), so the cells of `grid1.in` are the
  gmsh elements in file order.
The result is a `cases.Mesh`, written with `cases.write_grid`.
"""
from __future__ import annotations

from typing import Dict, List, Tuple

import numpy as np

from .cases import Mesh

SYSTEM_BC = {1: 4, 2: 3, 3: 1, 4: 5, 5: 2, 6: 6}  # readgmsh.f90:68-73
NODES_PER_TYPE = {1: 2, 2: 3, 3: 4, 15: 1}          # line, triangle, quadrangle, point


def _section(lines: List[str], name: str) -> Tuple[int, int]:
    a = lines.index(f"${name}")
    b = lines.index(f"$End{name}")
    return a + 1, b


def read_msh(path: str) -> Mesh:
    """A 2-D gmsh 4.1 ASCII mesh as a Mesh (1-based node ids, cells in file order)."""
    with open(path) as f:
        lines = [ln.strip() for ln in f]
    a, _ = _section(lines, "MeshFormat")
    version, filetype = lines[a].split()[:2]
    if not version.startswith("4.1") or filetype != "0":
        raise ValueError(f"{path}: gmsh 4.1 ASCII expected, got version {version} type {filetype}")
    # curves and their first physical tag (0: none)
    a, b = _section(lines, "Entities")
    npts, ncur, nsur, nvol = (int(x) for x in lines[a].split()[:4])
    curve_tag: Dict[int, int] = {}
    for ln in lines[a + 1 + npts:a + 1 + npts + ncur]:
        v = ln.split()
        tag, nphys = int(v[0]), int(v[7])
        curve_tag[tag] = int(v[8]) if nphys > 0 else 0
    # nodes (tags may be sparse: keep them and renumber densely in tag order)
    a, b = _section(lines, "Nodes")
    nblocks, nnodes = (int(x) for x in lines[a].split()[:2])
    tags = np.zeros(nnodes, dtype=np.int64)
    xyz = np.zeros((nnodes, 3))
    k, pos = 0, a + 1
    for _ in range(nblocks):
        _, _, param, n = (int(x) for x in lines[pos].split())
        if param:
            raise ValueError("parametric nodes are not supported")
        tags[k:k + n] = [int(x) for x in lines[pos + 1:pos + 1 + n]]
        xyz[k:k + n] = np.array([[float(x) for x in ln.split()[:3]] for ln in lines[pos + 1 + n:pos + 1 + 2 * n]])
        k += n
        pos += 1 + 2 * n
    order = np.argsort(tags)
    dense = {int(t): i + 1 for i, t in enumerate(tags[order])}
    coor = xyz[order, :2]
    # elements: 2-D cells in file order, boundary lines per physical tag
    a, b = _section(lines, "Elements")
    nblocks = int(lines[a].split()[0])
    cells: List[List[int]] = []
    edges: Dict[int, List[Tuple[int, int]]] = {}
    pos = a + 1
    for _ in range(nblocks):
        dim, etag, etype, n = (int(x) for x in lines[pos].split())
        npe = NODES_PER_TYPE.get(etype)
        if npe is None:
            raise ValueError(f"element type {etype} is not supported")
        for ln in lines[pos + 1:pos + 1 + n]:
            v = [dense[int(x)] for x in ln.split()[1:1 + npe]]
            if dim == 2:
                cells.append(v)
            elif dim == 1 and curve_tag.get(etag, 0) > 0:
                edges.setdefault(curve_tag[etag], []).append((v[0], v[1]))
        pos += 1 + n
    if any(len(c) != 3 for c in cells):
        raise ValueError("only triangular cells are written by this converter")
    boundaries = []
    for phys in sorted(edges):
        if phys not in SYSTEM_BC:
            raise ValueError(f"physical tag {phys} has no boundary code")
        boundaries.append((SYSTEM_BC[phys], np.array(edges[phys], dtype=np.int64)))
    return Mesh(coor=coor, cells=np.array(cells, dtype=np.int64), boundaries=boundaries, nx=0, ny=0)


def write_msh(path: str, mesh: Mesh, phys_of_bc: Dict[int, int]) -> None:
    """A Mesh as gmsh 4.1 ASCII (one surface, one curve entity per boundary
    group with the physical tag phys_of_bc[code]); for tests of read_msh."""
    nn = mesh.coor.shape[0]
    with open(path, "w") as f:
        f.write("$MeshFormat\n4.1 0 8\n$EndMeshFormat\n")
        f.write(f"$Entities\n0 {len(mesh.boundaries)} 1 0\n")
        for i, (code, _) in enumerate(mesh.boundaries):
            f.write(f"{i + 1} 0 0 0 0 0 0 1 {phys_of_bc[code]} 0\n")
        f.write(f"1 0 0 0 0 0 0 1 7 {len(mesh.boundaries)} " + " ".join(str(i + 1) for i in range(len(mesh.boundaries)))
                + "\n$EndEntities\n")
        f.write(f"$Nodes\n1 {nn} 1 {nn}\n2 1 0 {nn}\n")
        f.write("".join(f"{i + 1}\n" for i in range(nn)))
        f.write("".join(f"{float(x)!r} {float(y)!r} 0\n" for x, y in mesh.coor))
        f.write("$EndNodes\n")
        ne = sum(len(p) for _, p in mesh.boundaries) + mesh.cells.shape[0]
        f.write(f"$Elements\n{len(mesh.boundaries) + 1} {ne} 1 {ne}\n")
        tag = 1
        for i, (_, pairs) in enumerate(mesh.boundaries):
            f.write(f"1 {i + 1} 1 {len(pairs)}\n")
            for a, b in pairs:
                f.write(f"{tag} {a} {b}\n")
                tag += 1
        f.write(f"2 1 2 {mesh.cells.shape[0]}\n")
        for c in mesh.cells:
            f.write(f"{tag} {c[0]} {c[1]} {c[2]}\n")
            tag += 1
        f.write("$EndElements\n")
