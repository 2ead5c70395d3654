"""CPU oracle: numpy restatement of the reference's sweep semantics.

TEST INFRASTRUCTURE ONLY.  Nothing in the product path imports this package;
tests, ``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` use it
to check results.

It interprets the typed IR (shared front end) the way the reference's generated
C executes (xgrid/lang/generator.py):

* scalar statements run in program order with C typing: literals are ``double``
  (generator.py:393-394), arithmetic follows C's usual conversions, integer
  ``/`` truncates, ``%`` is C's remainder, ``x ** 2.0`` is ``x * x`` (what gcc makes of
  ``pow(x, 2.0)``, generator.py:377-383);
* every grid assignment is a sweep over the target's cells whose mask equals
  the assignment's ``boundary`` value (generator.py:289-304, 353-361); all values
  are computed from the state before the sweep and then stored, which is the
  two-phase semantics of implicit sweeps (generator.py:312-352) and equal to the
  reference's loop for every sweep whose cells do not read each other;
* neighbour addressing per overstep mode (generator.py:167-182): ``wrap`` and
  ``limit`` per axis; ``none`` is the row-major flattened offset, and a read that
  leaves the allocation returns 0 (the reference reads outside its array there);
* time level of a stencil = |time offset| (generator.py:424-432).

Grids use C order for every shape.  For square 2-D grids this is the
reference's addressing; for non-square and 3-D grids the reference's own
indexing is wrong (it strides by the wrong extent), and the oracle follows the
intended C-order semantics.
"""
from __future__ import annotations

import numpy as np

from xgrid_gb300 import ir
from xgrid_gb300.types import (Boolean, Floating, GridType, Integer, Pointer, Structure, Void)

_NP = {"bool": np.bool_, "int8_t": np.int8, "int16_t": np.int16, "int": np.int32, "int32_t": np.int32,
       "int64_t": np.int64, "float": np.float32, "double": np.float64}
_RANK = {"bool": 0, "int8_t": 1, "int16_t": 2, "int": 3, "int32_t": 3, "int64_t": 4}


def ctype_of_type(t) -> str:
    if isinstance(t, Boolean):
        return "bool"
    if isinstance(t, Integer):
        return {1: "int8_t", 2: "int16_t", 4: "int", 8: "int64_t"}[t.width_bytes]
    if isinstance(t, Floating):
        return "float" if t.width_bytes == 4 else "double"
    if isinstance(t, Structure):
        return "struct"
    if isinstance(t, Pointer):
        return ctype_of_type(t.element)
    raise TypeError(t)


def usual(a: str, b: str) -> str:
    if "double" in (a, b):
        return "double"
    if "float" in (a, b):
        return "float"
    return "int64_t" if max(_RANK.get(a, 3), _RANK.get(b, 3)) == 4 else "int"


class Struct:
    """A struct value (dataclass instance restated as named fields)."""

    def __init__(self, stype: Structure, fields: dict) -> None:
        self.stype = stype
        self.fields = fields

    @classmethod
    def from_value(cls, stype: Structure, value) -> "Struct":
        out = {}
        for name, t in stype.elements:
            v = getattr(value, name)
            out[name] = Struct.from_value(t, v) if isinstance(t, Structure) else cast(np.asarray(v), ctype_of_type(t))
        return cls(stype, out)

    def to_value(self):
        args = []
        for name, t in self.stype.elements:
            v = self.fields[name]
            args.append(v.to_value() if isinstance(v, Struct) else v.item())
        return self.stype.dataclass(*args)


def cast(v, ct: str):
    dt = _NP[ct]
    if isinstance(v, np.ndarray) or np.isscalar(v) or isinstance(v, np.generic):
        a = np.asarray(v)
        if a.dtype == dt:
            return a
        if np.issubdtype(a.dtype, np.floating) and np.issubdtype(dt, np.integer):
            with np.errstate(invalid="ignore"):
                return np.trunc(a).astype(dt)
        return a.astype(dt)
    raise TypeError(f"cannot cast {type(v)}")


class _Break(Exception):
    pass


class _Continue(Exception):
    pass


class _Return(Exception):
    def __init__(self, value):
        self.value = value


class Interpreter:
    """Executes one operator's IR."""

    def __init__(self, defn: ir.Definition, overstep: str, before_sweep=None) -> None:
        self.defn = defn
        self.overstep = overstep
        self.before_sweep = before_sweep  # callable(stmt, env) run before every grid sweep

    # ----------------------------------------------------------- types
    def ctype(self, e) -> str:
        if isinstance(e, ir.Constant):
            if isinstance(e.value, bool):
                return "int"
            return "int" if isinstance(e.value, int) else "double"
        if isinstance(e, (ir.Identifier, ir.Stencil, ir.Access, ir.Call, ir.Cast)):
            if isinstance(e.type, Structure):
                return "struct"
            return ctype_of_type(e.type)
        if isinstance(e, ir.GridInfo):
            return "int"
        if isinstance(e, ir.Unary):
            return "int" if e.operator is ir.UnaryOperator.Not else usual(self.ctype(e.right), "int")
        if isinstance(e, ir.Condition):
            a, b = self.ctype(e.body), self.ctype(e.orelse)
            return a if a == b else usual(a, b)
        if isinstance(e, ir.Binary):
            if e.operator.is_compare() or e.operator.is_logic():
                return "int"
            if e.operator is ir.BinaryOperator.Pow:
                return "double" if isinstance(e.type, Floating) and e.type.width_bits == 64 else "float"
            return usual(self.ctype(e.left), self.ctype(e.right))
        raise TypeError(e)

    # ------------------------------------------------------ expressions
    def eval(self, e, env: dict, cells=None):
        if isinstance(e, ir.Constant):
            if isinstance(e.value, bool):
                return np.asarray(1 if e.value else 0, dtype=np.int32)
            return np.asarray(e.value, dtype=np.int32 if isinstance(e.value, int) else np.float64)
        if isinstance(e, ir.Identifier):
            return env[e.variable.name]
        if isinstance(e, ir.Access):
            base = self.eval(e.value, env, cells)
            if isinstance(base, Struct):
                return base.fields[e.attribute]
            return np.asarray(base[e.attribute])  # structured array of a struct grid
        if isinstance(e, ir.Stencil):
            return self.load(e, env, cells)
        if isinstance(e, ir.GridInfo):
            g = env[e.variable.name]
            if e.info == "dimension":
                return np.asarray(len(g.shape), dtype=np.int32)
            return np.asarray(g.shape[int(self.eval(e.dimension, env, cells))], dtype=np.int32)
        if isinstance(e, ir.Cast):
            return cast(self.eval(e.value, env, cells), ctype_of_type(e.type))
        if isinstance(e, ir.Unary):
            v = self.eval(e.right, env, cells)
            if e.operator is ir.UnaryOperator.Not:
                return np.logical_not(v).astype(np.int32)
            ct = self.ctype(e)
            v = cast(v, ct)
            return -v if e.operator is ir.UnaryOperator.Neg else v
        if isinstance(e, ir.Condition):
            c = self.eval(e.condition, env, cells)
            ct = self.ctype(e)
            a = cast(self.eval(e.body, env, cells), ct)
            b = cast(self.eval(e.orelse, env, cells), ct)
            return np.where(np.asarray(c) != 0, a, b).astype(_NP[ct])
        if isinstance(e, ir.Binary):
            return self.binary(e, env, cells)
        if isinstance(e, ir.Call):
            return self.call(e, env, cells)
        raise TypeError(type(e).__name__)

    def binary(self, e: ir.Binary, env, cells):
        op = e.operator
        B = ir.BinaryOperator
        if op in (B.And, B.Or):
            a = np.asarray(self.eval(e.left, env, cells)) != 0
            b = np.asarray(self.eval(e.right, env, cells)) != 0
            return (np.logical_and(a, b) if op is B.And else np.logical_or(a, b)).astype(np.int32)
        if op is B.Pow:
            ct = self.ctype(e)
            base = cast(self.eval(e.left, env, cells), ct)
            r = e.right
            k = None
            if isinstance(r, ir.Constant) and not isinstance(r.value, bool) and r.value in (2, 1, 0, -1):
                k = float(r.value)
            if k == 2.0:
                return base * base
            if k == 1.0:
                return base
            if k == 0.0:
                return np.ones_like(base)
            if k == -1.0:
                return _NP[ct](1) / base
            ex = cast(self.eval(r, env, cells), ct)
            with np.errstate(all="ignore"):
                return np.power(base, ex)
        a = self.eval(e.left, env, cells)
        b = self.eval(e.right, env, cells)
        if op.is_compare():
            ct = usual(self.ctype(e.left), self.ctype(e.right))
            a, b = cast(a, ct), cast(b, ct)
            f = {B.Eq: np.equal, B.Neq: np.not_equal, B.Gt: np.greater, B.Ge: np.greater_equal,
                 B.Lt: np.less, B.Le: np.less_equal}[op]
            return f(a, b).astype(np.int32)
        ct = self.ctype(e)
        a, b = cast(a, ct), cast(b, ct)
        with np.errstate(all="ignore"):
            if op is B.Add:
                return a + b
            if op is B.Sub:
                return a - b
            if op is B.Mul:
                return a * b
            if op is B.Div:
                if ct in ("float", "double"):
                    return a / b
                bs = np.where(b == 0, 1, b)
                q = np.abs(a) // np.abs(bs)
                return np.where(b == 0, 0, q * np.sign(a) * np.sign(bs)).astype(_NP[ct])
            if op is B.Mod:
                bs = np.where(b == 0, 1, b)
                return np.where(b == 0, 0, np.fmod(a, bs)).astype(_NP[ct])
        raise TypeError(op)

    def call(self, e: ir.Call, env, cells):
        args = [self.eval(a, env, cells) for a in e.arguments]
        if isinstance(e.operator, ir.Constructor):
            st = e.operator.type
            return Struct(st, {n: (v if isinstance(v, Struct) else cast(v, ctype_of_type(t)))
                               for (n, t), v in zip(st.elements, args)})
        op = e.operator
        if op.mode == "external":
            raise NotImplementedError(f"external '{op.name}' has no CPU restatement")
        defn = op.ir
        sub = Interpreter(defn, self.overstep)
        arrays = [a for a in args if isinstance(a, np.ndarray) and a.ndim > 0]
        if not arrays:
            return sub.run_function(args)
        shape = np.broadcast(*arrays).shape
        out = None
        for idx in np.ndindex(shape):
            scalar_args = [a[idx] if isinstance(a, np.ndarray) and a.ndim > 0 else a for a in args]
            r = sub.run_function([np.asarray(x) if not isinstance(x, Struct) else x for x in scalar_args])
            if out is None:
                out = np.empty(shape, dtype=np.asarray(r).dtype)
            out[idx] = r
        return out

    def run_function(self, args: list):
        env = {}
        for (name, t), v in zip(self.defn.signature.arguments, args):
            env[name] = v if isinstance(v, Struct) else cast(v, ctype_of_type(t))
        try:
            self.block(self.defn.body, env)
        except _Return as r:
            v = r.value
            rt = self.defn.signature.return_type
            if v is None or isinstance(rt, Void):
                return None
            return v if isinstance(v, Struct) else cast(v, ctype_of_type(rt))
        return None

    # ------------------------------------------------------------ grids
    def load(self, e: ir.Stencil, env, cells):
        if cells is None:
            raise Exception(f"Unable to perform load operation to grid '{e.variable.name}' without stencil context")
        g = env[e.variable.name]
        level = abs(e.time_offset)
        flat = g.levels[level].reshape(-1)
        idx = self.address(cells, e.space_offset, g.shape)
        valid = idx >= 0
        out = flat[np.where(valid, idx, 0)]
        if not valid.all():
            out = np.where(valid, out, np.zeros((), dtype=flat.dtype))
        return out

    def address(self, cells, offset, shape):
        """Linear index of every domain cell + ``offset`` in a grid of ``shape``."""
        coords = cells
        nd = len(shape)
        if self.overstep == "none":
            t = np.zeros(coords[0].shape, dtype=np.int64)
            for d in range(nd):
                t = t * shape[d] + (coords[d] + offset[d])
            total = int(np.prod(shape))
            return np.where((t >= 0) & (t < total), t, -1)
        t = np.zeros(coords[0].shape, dtype=np.int64)
        for d in range(nd):
            c = coords[d] + offset[d]
            c = np.mod(c, shape[d]) if self.overstep == "wrap" else np.clip(c, 0, shape[d] - 1)
            t = t * shape[d] + c
        return t

    def sweep(self, stmt: ir.Assignment, env):
        if self.before_sweep is not None:  # e.g. a slab decomposition refreshing halo rows
            self.before_sweep(stmt, env)
        target: ir.Stencil = stmt.terminal
        g = env[target.variable.name]
        cells = tuple(c.reshape(-1).astype(np.int64) for c in np.indices(g.shape))
        mask = g.boundary.reshape(-1) == target.boundary_mask
        value = self.eval(stmt.value, env, cells)
        dst = g.levels[abs(target.time_offset)].reshape(-1)
        value = np.broadcast_to(np.asarray(value), mask.shape)
        if g.levels[0].dtype.names is None:
            value = cast(value, ctype_of_type(g.element))
        idx = self.address(cells, target.space_offset, g.shape)
        sel = mask & (idx >= 0)
        dst[idx[sel]] = value[sel]

    # ------------------------------------------------------- statements
    def block(self, stmts, env):
        for s in stmts:
            self.stmt(s, env)

    def stmt(self, s, env):
        if isinstance(s, ir.Assignment):
            if isinstance(s.terminal, ir.Stencil):
                self.sweep(s, env)
                return
            v = self.eval(s.value, env)
            self.store(s.terminal, v, env)
        elif isinstance(s, ir.Return):
            raise _Return(None if s.value is None else self.eval(s.value, env))
        elif isinstance(s, ir.Break):
            raise _Break()
        elif isinstance(s, ir.Continue):
            raise _Continue()
        elif isinstance(s, ir.Evaluation):
            self.eval(s.value, env)
        elif isinstance(s, ir.If):
            self.block(s.body if self.eval(s.condition, env) != 0 else s.orelse, env)
        elif isinstance(s, ir.While):
            while self.eval(s.condition, env) != 0:
                try:
                    self.block(s.body, env)
                except _Break:
                    break
                except _Continue:
                    continue
        elif isinstance(s, ir.For):
            ct = ctype_of_type(s.variable.type)
            env[s.variable.name] = cast(self.eval(s.start, env), ct)
            while env[s.variable.name] < self.eval(s.end, env):
                try:
                    self.block(s.body, env)
                except _Break:
                    break
                except _Continue:
                    pass
                env[s.variable.name] = cast(env[s.variable.name] + self.eval(s.step, env), ct)
        elif isinstance(s, ir.Inline):
            raise NotImplementedError("inline C has no CPU restatement")
        else:
            raise TypeError(type(s).__name__)

    def store(self, t, v, env):
        if isinstance(t, ir.Identifier):
            env[t.variable.name] = v if isinstance(v, Struct) else cast(v, ctype_of_type(t.type))
        elif isinstance(t, ir.Access):
            base = self.eval(t.value, env)
            base.fields[t.attribute] = v if isinstance(v, Struct) else cast(v, ctype_of_type(t.type))
        else:
            raise TypeError(type(t).__name__)

    def run_kernel(self, args: list):
        env = {}
        for (name, t), v in zip(self.defn.signature.arguments, args):
            if isinstance(t, GridType):
                env[name] = v
            elif isinstance(t, Structure):
                env[name] = Struct.from_value(t, v)
            else:
                env[name] = cast(np.asarray(v), ctype_of_type(t))
        for name, var in self.defn.scope.items():
            if name not in env:
                env[name] = None
        try:
            self.block(self.defn.body, env)
        except _Return as r:
            rt = self.defn.signature.return_type
            if r.value is None or isinstance(rt, Void):
                return None
            if isinstance(r.value, Struct):
                return r.value.to_value()
            return cast(r.value, ctype_of_type(rt)).item()
        return None


def depth_of(defn: ir.Definition) -> int:
    """Levels a kernel needs: max |time offset| + 1 (generator.py:106-108, 428)."""
    d = 0
    for n in ir.walk(defn.body):
        if isinstance(n, ir.Stencil):
            d = max(d, abs(n.time_offset))
    return d + 1
