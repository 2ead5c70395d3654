"""Parser and typing: the reference's acceptance rules and error messages
(xgrid/lang/parser.py), checked without a GPU."""
import dataclasses

import pytest

import xgrid
from xgrid_gb300 import ir
from xgrid_gb300.operator import Operator
from xgrid_gb300.types import Floating, GridType, Integer


def parse(fn):
    return Operator(fn, "kernel", fn.__name__).ir


@pytest.fixture(autouse=True)
def _init():
    xgrid.init(precision="double", cacheroot="/tmp/xgfe")


def k_mixed_types(u: xgrid.grid[float, 2]) -> None:
    u[0, 0] = 2 * u[0, 0]


def k_bad_subscript(u: xgrid.grid[float, 2], i: int) -> None:
    u[0, 0] = u[i, 0]


def k_wrong_rank(u: xgrid.grid[float, 2]) -> None:
    u[0, 0] = u[0]


def k_no_annotation(u) -> None:
    pass


def k_no_return(u: xgrid.grid[float, 2]):
    pass


def k_load_outside(u: xgrid.grid[float, 2]) -> float:
    return u[0, 0]


def k_augassign(u: xgrid.grid[float, 2]) -> None:
    u[0, 0] += 1.0


@pytest.mark.parametrize("fn,msg", [
    (k_mixed_types, "Incompatible binary operator"),
    (k_bad_subscript, "Incompatible subscript"),
    (k_wrong_rank, "Incompatible subscript length"),
    (k_no_annotation, "requires type annotation"),
    (k_no_return, "Invalid return type"),
    (k_augassign, "Augmented assignment to a grid"),
])
def test_rejected_programs(fn, msg):
    with pytest.raises(Exception) as e:
        parse(fn)
    assert msg in " ".join(map(str, e.value.args))


def test_load_outside_a_sweep_is_rejected_by_the_generator():
    from xgrid_gb300.codegen import CudaGenerator
    from xgrid_gb300.config import get_config
    with pytest.raises(Exception, match="without stencil context"):
        CudaGenerator(Operator(k_load_outside, "kernel", "k_load_outside"), get_config()).generate()


def k_time_levels(u: xgrid.grid[float, 1], v: xgrid.grid[float, 1]) -> None:
    with xgrid.boundary(3):
        u[0] = u[1] + v[-1][0] + u[0][-2]


def test_stencil_times_offsets_masks():
    d = parse(k_time_levels)
    a = d.body[0]
    assert isinstance(a.terminal, ir.Stencil) and a.terminal.time_offset == 0 and a.terminal.boundary_mask == 3
    loads = ir.stencils(a.value)
    assert [(s.variable.name, s.time_offset, s.space_offset, s.boundary_mask) for s in loads] == \
        [("u", -1, (1,), 3), ("v", 0, (-1,), 3), ("u", -2, (0,), 3)]


def k_pow_types(a: int, x: float) -> float:
    return x ** 2.0 + a ** a


def test_pow_typing_follows_the_reference():
    d = parse(k_pow_types)
    e = d.body[0].value
    assert e.left.type == Floating(8) and e.right.type == Floating(8)  # precision double


def test_float_width_follows_precision():
    xgrid.init(precision="float", cacheroot="/tmp/xgfe")
    d = parse(k_time_levels)
    assert d.signature.arguments[0][1] == GridType(Floating(4), 1)
    xgrid.init(precision="double", cacheroot="/tmp/xgfe")
    assert parse(k_time_levels).signature.arguments[0][1] == GridType(Floating(8), 1)


@dataclasses.dataclass
class Pair:
    a: int
    b: int


def k_struct(p: Pair) -> int:
    q = Pair(p.b, p.a)
    return q.a - q.b


def test_struct_constructor_and_access():
    d = parse(k_struct)
    assert d.scope["q"].type.name == "Pair"
    assert d.signature.return_type == Integer(4)


def test_grid_api_on_host():
    g = xgrid.Grid((4, 6), float)
    g.now[...] = 1.5
    g.boundary[0, :] = 1
    g.fill(g.now * 2, time=0)
    assert (g.read(0) == 3.0).all()
    assert g.dimension == 2 and g.boundary.dtype.name == "int32"
    g._op_invoke(3, True)
    assert g.time == 3


@pytest.mark.parametrize("kw,msg", [
    ({"overstep": "mirror"}, "Invalid overstep"),
    ({"precision": "half"}, "Invalid precision"),
    ({"mixed": "fp8"}, "Invalid mixed precision"),
    ({"opt_level": 5}, "Invalid opt_level"),
    ({"mixed_temporal": 17}, "Invalid mixed_temporal"),
    ({"mixed_rows": 12}, "Invalid mixed_rows"),
    ({"int_adds": -1}, "Invalid int_adds"),
])
def test_invalid_configuration_is_rejected(kw, msg):
    with pytest.raises(Exception) as e:
        xgrid.init(cacheroot="/tmp/xgfe", **kw)
    assert msg in str(e.value)


def test_configuration_defaults_and_flags():
    from xgrid_gb300.config import get_config
    xgrid.init(cacheroot="/tmp/xgfe")
    c = get_config()
    assert (c.precision, c.overstep, c.mixed, c.persistent, c.fuse, c.graph) == ("float", "none", None, False, True,
                                                                                  True)
    assert "--fmad=false" in c.nvcc_flags
    xgrid.init(cacheroot="/tmp/xgfe", exact=False, precision="double", persistent=True)
    c = get_config()
    assert "--fmad=false" not in c.nvcc_flags and c.fsize == 8 and c.persistent


@pytest.mark.parametrize("shape,msg", [((0, 4), "extents must be positive"), ((2, 2, 2, 2), "not supported")])
def test_grid_shapes_rejected(shape, msg):
    with pytest.raises(Exception) as e:
        xgrid.Grid(shape, float)
    assert msg in str(e.value)


def test_grid_level_rotation_follows_the_reference():
    """tick moves the last level to the front (xgrid/xgrid/__init__.py:49-54)."""
    g = xgrid.Grid(5, float)
    g._op_invoke(3, False)
    for i in range(3):
        g.fill(g.now * 0 + i, time=-i)
    assert [float(g._data[i][0]) for i in range(3)] == [0.0, 1.0, 2.0]
    g._op_invoke(3, True)
    assert [float(g._data[i][0]) for i in range(3)] == [2.0, 0.0, 1.0]
    # fill beyond the current depth extends the level list
    g.fill(g.now * 0 + 7, time=4)
    assert g.time == 5 and float(g._data[4][0]) == 7.0


def test_grid_read_is_a_copy_and_now_is_the_level():
    g = xgrid.Grid((3, 3), float)
    g.now[...] = 2.0
    r = g.read(0)
    r[...] = 5.0
    assert (g.now == 2.0).all()
    g[1, 1] = 9.0
    assert g.now[1, 1] == 9.0 and g[1, 1] == 9.0
