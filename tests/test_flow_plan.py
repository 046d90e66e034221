"""The dataflow LU-SGS plan (host side, no GPU): the level order of both
sweeps, the per-block passes and their cross-block dependencies that rc_init
builds for k_lusgs_flow, checked by rc_flow_plan_check on nozzle meshes in the
natural, colored and random cell orders, and the blocks' protocol run in
synchronous steps to its end (no deadlock; at least as many steps as levels)."""
import numpy as np
import pytest

import rocketcombustor_gb300 as rc
from rocketcombustor_gb300.cases import nozzle_mesh


def _graph(nx, ny, order, seed=3):
    cells = nozzle_mesh(nx, ny, seed, order).cells
    ne = cells.shape[0]
    cother = -np.ones((ne, 4), np.int32)
    first = {}
    for c, tri in enumerate(cells):
        for q, (a, b) in enumerate(((tri[0], tri[1]), (tri[1], tri[2]), (tri[2], tri[0]))):
            k = (min(a, b), max(a, b))
            if k in first:
                o, oq = first.pop(k)
                cother[c, q] = o
                cother[o, oq] = c
            else:
                first[k] = (c, q)
    return np.full(ne, 3, np.int32), cother


@pytest.mark.parametrize("nx,ny,order,nblocks", [(24, 6, "natural", 152), (24, 6, "natural", 4),
                                                 (100, 20, "natural", 152), (100, 20, "colored", 152),
                                                 (100, 20, "random", 152), (100, 20, "natural", 1)])
def test_plan_is_consistent_and_runs_to_the_end(nx, ny, order, nblocks):
    nface, cother = _graph(nx, ny, order)
    ne = nface.shape[0]
    st = rc.flow_plan_check(nface, cother, nblocks)
    assert st["passes_fwd"] >= st["levels_fwd"] and st["passes_bwd"] >= st["levels_bwd"]
    assert st["passes_fwd"] <= ne and st["passes_bwd"] <= ne
    # the steps are at least the longest dependency chain through both sweeps
    # and at most one pass per step
    assert st["levels_fwd"] + st["levels_bwd"] <= st["steps"] <= st["passes_fwd"] + st["passes_bwd"]
    assert st["cells_per_block"] == -(-ne // nblocks)
    if nblocks == 1:
        assert st["deps"] == 0  # one block: every dependency is inside it


@pytest.mark.parametrize("nx,ny", [(100, 20), (300, 50)])
def test_natural_order_plan_adds_nothing_to_the_critical_path(nx, ny):
    """The natural order of a nozzle (columns downstream, bottom to top inside a
    column) split over 152 blocks: with equal pass times the blocks' protocol
    ends in exactly as many steps as there are levels in the two sweeps, and a
    pass waits for at most two passes of other blocks."""
    nface, cother = _graph(nx, ny, "natural")
    st = rc.flow_plan_check(nface, cother, 152)
    assert st["levels_fwd"] == st["levels_bwd"]
    assert st["max_deps"] <= 2
    assert st["steps"] == st["levels_fwd"] + st["levels_bwd"]


@pytest.mark.parametrize("nx,ny,order", [(24, 6, "natural"), (100, 20, "colored"), (100, 20, "random"),
                                         (3000, 8, "natural"), (9000, 4, "natural")])
@pytest.mark.parametrize("groups", [1, 2])
@pytest.mark.parametrize("nvar", [4, 7])
def test_compact_plan_is_consistent(nx, ny, order, groups, nvar):
    """The compact plans of k_lusgs_flowc (groups of at most 128 / nvar cells
    and 32 active pairs, each group listing exactly its cells' active pairs)
    pass every check and need no more passes than the 8-position plan of as
    many groups; on the long, thin nozzle with about 13 cells of a level per
    block two compact groups end in as many steps as there are levels, and
    with about 39 they need more passes with one group than with two."""
    nface, cother = _graph(nx, ny, order)
    st = rc.flow_plan_check(nface, cother, 152, groups=groups, compact=True, nvar=nvar)
    old = rc.flow_plan_check(nface, cother, 152, groups=groups)
    assert st["passes_fwd"] <= old["passes_fwd"] and st["passes_bwd"] <= old["passes_bwd"]
    assert st["levels_fwd"] + st["levels_bwd"] <= st["steps"] <= st["passes_fwd"] + st["passes_bwd"]
    if (nx, ny, groups) == (3000, 8, 2):
        assert st["steps"] == st["levels_fwd"] + st["levels_bwd"]
    if (nx, ny) == (9000, 4) and groups == 2:
        one = rc.flow_plan_check(nface, cother, 152, groups=1, compact=True, nvar=nvar)
        assert st["passes_fwd"] < one["passes_fwd"]


def test_compact_plan_of_the_benchmark_mesh_has_one_group_per_level():
    """The 2,000,000-cell benchmark nozzle (2500 x 400): a block holds at most
    17 cells (26 active pairs) of a level, within one group of the
    four-species build (18 cells), so the compact plan with one group ends
    in as many steps as there are levels."""
    nface, cother = _graph(2500, 400, "natural")
    st = rc.flow_plan_check(nface, cother, 152, groups=1, compact=True, nvar=7)
    assert st["steps"] == st["levels_fwd"] + st["levels_bwd"] == 2402


def test_bad_arguments_are_refused():
    nface, cother = _graph(24, 6, "natural")
    bad = cother.copy()
    bad[0, 0] = nface.shape[0] + 5  # out of range
    with pytest.raises(rc.RcError):
        rc.flow_plan_check(nface, bad, 8)
    with pytest.raises(rc.RcError):
        rc.flow_plan_check(nface, cother, 0)
    with pytest.raises(rc.RcError):
        rc.flow_plan_check(nface, cother, 8, groups=3, compact=True)
    with pytest.raises(rc.RcError):
        rc.flow_plan_check(nface, cother, 8, groups=1, compact=True, nvar=2)
