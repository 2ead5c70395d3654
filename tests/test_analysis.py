"""Launch grouping rules on the CPU: which consecutive sweeps one launch may run
(tile by tile, phases separated by __syncthreads).  A main sweep may not read,
at a nonzero offset, a buffer version another sweep of its group writes (another
tile may not have written it yet); a sweep storing at an offset runs alone; a
main sweep after boundary sweeps opens a new group; boundary sweeps that read a
buffer written in the group at an offset get a tile-locality check; implicit
sweeps write a new version (the scratch buffer); ``fuse=False`` gives one launch
per sweep."""
import xgrid
from xgrid_gb300.codegen import CudaGenerator
from xgrid_gb300.config import get_config
from xgrid_gb300.operator import Operator

g2 = xgrid.grid[float, 2]


def _groups(fn, **cfg):
    xgrid.init(precision="double", cacheroot="/tmp/xgcg", opt_level=3, **cfg)
    gen = CudaGenerator(Operator(fn, "kernel", fn.__name__), get_config())
    gen.generate()
    return [em.g for em in gen.group_emitters]


def _shape(groups):
    return [[("main" if s.is_main else f"bnd{s.mask}") + ("*" if s.implicit else "") for s in g.sweeps]
            for g in groups]


def offset_read_of_fresh_write(a: g2, b: g2) -> None:
    a[0, 0] = b[0, 0] + 1.0
    b[0, 0] = a[0, 1][0] * 2.0


def same_cell_read_of_fresh_write(a: g2, b: g2) -> None:
    a[0, 0] = b[0, 0] + 1.0
    b[0, 0] = a[0, 0][0] * 2.0


def relax(p: g2, f: g2) -> None:
    p[0, 0] = 0.25 * (p[1, 0][0] + p[-1, 0][0] + p[0, 1][0] + p[0, -1][0] - f[0, 0][0])
    with xgrid.boundary(1):
        p[0, 0] = p[0, 1][0]
    with xgrid.boundary(2):
        p[0, 0] = 0.0


def offset_store(a: g2, b: g2) -> None:
    a[0, 0] = b[0, 0]
    a[0, 1] = b[0, 0] * 0.5
    b[0, 0] = a[0, 0]


def main_after_boundary(a: g2, b: g2) -> None:
    a[0, 0] = b[0, 0] + 1.0
    with xgrid.boundary(1):
        a[0, 0] = 0.0
    b[0, 0] = b[0, 0] * 2.0


def implicit_after_write(p: g2, q: g2) -> None:
    p[0, 0] = q[0, 0]
    p[0, 0] = 0.5 * (p[1, 0][0] + p[-1, 0][0])


def store_at_a_time_offset(q: g2) -> None:
    q[0, 0][-1] = 0.5 * (q[0, 1][0] + q[0, -1][0])


def test_offset_read_of_a_fresh_write_splits():
    assert _shape(_groups(offset_read_of_fresh_write)) == [["main"], ["main"]]


def test_same_cell_read_of_a_fresh_write_fuses():
    assert _shape(_groups(same_cell_read_of_fresh_write)) == [["main", "main"]]


def test_implicit_sweep_and_boundary_phases_fuse_with_a_locality_check():
    (g,) = _groups(relax)
    assert _shape([g]) == [["main*", "bnd1", "bnd2"]]
    main, b1, b2 = g.sweeps
    assert (main.read_version_of_target, main.write_version) == (0, 1)
    # the boundary phases work on the new version in place
    assert b1.write_version == 1 and b2.write_version == 1
    # boundary(1) reads p[0, 1] of the version the group writes: tile-local check needed
    assert g.local_checks == [(1, [(0, 0, 1)])]


def test_offset_store_runs_alone():
    shape = _shape(_groups(offset_store))
    assert ["main"] in shape and len(shape) == 3


def test_main_after_boundary_opens_a_group():
    assert _shape(_groups(main_after_boundary)) == [["main", "bnd1"], ["main"]]


def test_implicit_sweep_after_a_write_of_its_input_splits():
    shape = _shape(_groups(implicit_after_write))
    assert shape == [["main"], ["main*"]]


def test_store_at_a_time_offset_is_rejected_like_the_reference():
    """``g[o][t] = ...`` is a load in the target position: the reference dies with
    this message (xgrid/lang/generator.py:62-65), so every sweep writes level 0."""
    import pytest
    with pytest.raises(Exception, match="Unable to perform load operation to grid 'q' without stencil context"):
        _groups(store_at_a_time_offset)


def test_no_fusion_gives_one_launch_per_sweep():
    assert _shape(_groups(relax, fuse=False)) == [["main*"], ["bnd1"], ["bnd2"]]
    assert _shape(_groups(same_cell_read_of_fresh_write, fuse=False)) == [["main"], ["main"]]
