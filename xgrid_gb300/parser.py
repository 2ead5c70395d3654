"""Front end: the Python source of an ``@xgrid.kernel`` / ``@xgrid.function``
body becomes the typed IR of ``ir.py``.

What is accepted, how it is typed and the text of every diagnostic are those of
the reference front end (xgrid/lang/parser.py:54-641), because a drop-in
replacement must accept and reject the same programs with the same messages:

* ``g[o0, ..., oN-1]`` is a stencil access with integer-literal offsets; a load
  without a time subscript reads time -1, a store writes time 0, ``g[...][t]``
  names time ``t`` (parser.py:456-525);
* ``with xgrid.boundary(k):`` masks the stencils written inside it, ``with
  xgrid.c():`` turns string statements into inline source, ``import a.b``
  becomes ``#include "a/b.h"`` (parser.py:200-235, 328-337);
* arithmetic needs operands of one numeric type; ``**`` is FP64 when the left
  operand is FP64 and ``float`` otherwise; a comparison chain compares its first
  operand with each of the others (parser.py:365-414);
* global names fold to constants; calls resolve kernels' helper functions,
  externals (with their type-check override), dataclass constructors and
  methods, ``typing.cast`` and the built-ins ``shape``/``dimension``
  (parser.py:548-641).

Organisation (independent of the reference's visitor): ``_Source`` holds the
parsed function, ``Scope`` the kernel's symbols and the current pragma state,
``_Lookup`` resolves Python-side names, the type rules are plain functions, and
``Parser`` dispatches statements and expressions through rule tables whose
handlers always return lists of statements / one expression.  Every error goes
through ``Logger.dead`` and is raised as ``Exception``.
"""
from __future__ import annotations

import ast
import dataclasses
import inspect
import struct
import textwrap
import typing
from typing import NoReturn

from . import ir
from .config import get_config
from .log import Logger
from .types import (BaseType, Boolean, Floating, GridType, Integer, Number, Pointer,
                    Reference, Structure, Value, Void, parse_annotation)

INT = struct.calcsize("i")
DOUBLE = struct.calcsize("d")

UNARY_OPS = {ast.UAdd: ir.UnaryOperator.Pos, ast.USub: ir.UnaryOperator.Neg, ast.Not: ir.UnaryOperator.Not}
ARITH_OPS = {ast.Add: ir.BinaryOperator.Add, ast.Sub: ir.BinaryOperator.Sub, ast.Mult: ir.BinaryOperator.Mul,
             ast.Div: ir.BinaryOperator.Div, ast.Pow: ir.BinaryOperator.Pow, ast.Mod: ir.BinaryOperator.Mod}
COMPARE_OPS = {ast.Eq: ir.BinaryOperator.Eq, ast.NotEq: ir.BinaryOperator.Neq, ast.Gt: ir.BinaryOperator.Gt,
               ast.GtE: ir.BinaryOperator.Ge, ast.Lt: ir.BinaryOperator.Lt, ast.LtE: ir.BinaryOperator.Le}
LOGIC_OPS = {ast.And: ir.BinaryOperator.And, ast.Or: ir.BinaryOperator.Or}


# ----------------------------------------------------------------- type rules
def int_literal(node) -> int | None:
    """``k`` or ``-k`` for an integer literal ``k`` (the only legal offsets), else None."""
    negate = isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub)
    leaf = node.operand if negate else node
    if isinstance(leaf, ast.Constant) and type(leaf.value) is int:
        return -leaf.value if negate else leaf.value
    return None


def literal_type(value) -> BaseType | None:
    """DSL type of a Python constant: ``int`` is a C int, ``float`` the configured
    precision, ``bool`` a C bool; anything else has none."""
    return {int: Integer(INT), float: Floating(get_config().fsize), bool: Boolean()}.get(type(value))


def arithmetic_type(op: ir.BinaryOperator, left: BaseType, right: BaseType) -> BaseType | None:
    """Result type of ``left op right``, or None when the operands do not combine."""
    if not (isinstance(left, Number) and isinstance(right, Number)) or left != right:
        return None
    if op is ir.BinaryOperator.Pow:
        wide = isinstance(left, Floating) and left.width_bits == 64
        return Floating(DOUBLE if wide else get_config().fsize)
    return left


def unary_accepts(op: ir.UnaryOperator, operand: BaseType) -> bool:
    if op is ir.UnaryOperator.Not:
        return isinstance(operand, Boolean)
    return isinstance(operand, Number)


def ctx_of(node) -> str:
    return "load" if isinstance(node, ast.Load) else "store"


# ------------------------------------------------------------------ plumbing
@dataclasses.dataclass
class _Source:
    """The function's AST with line numbers of its file."""

    file: str
    tree: ast.FunctionDef

    @classmethod
    def of(cls, func) -> "_Source":
        file = inspect.getsourcefile(func) or "<unknown>"
        lines, first = inspect.getsourcelines(func)
        tree = ast.parse(textwrap.dedent("".join(lines)), file).body[0]
        ast.increment_lineno(tree, first)
        return cls(file, tree)


@dataclasses.dataclass
class Scope:
    """Symbols of the body and the pragma state at the current statement."""

    symbols: dict = dataclasses.field(default_factory=dict)
    regions: list = dataclasses.field(default_factory=list)  # kernel/function, if, while, c
    mask: int = 0                                            # active ``boundary(k)``
    includes: list = dataclasses.field(default_factory=list)

    @property
    def region(self) -> str:
        return self.regions[-1]


class _Lookup:
    """Python-side names: the function's globals, captured closure values and
    the built-in type names, followed through attribute chains."""

    def __init__(self, func) -> None:
        self.table = dict(func.__globals__)
        self.table.update({"int": int, "float": float, "bool": bool})
        try:
            self.table.update(inspect.getclosurevars(func).nonlocals)
        except (TypeError, ValueError):
            pass

    def chain(self, node) -> list | None:
        """``a.b.c`` -> ["a", "b", "c"], None for anything that is not a name chain."""
        parts = []
        while isinstance(node, ast.Attribute):
            parts.append(node.attr)
            node = node.value
        if not isinstance(node, ast.Name):
            return None
        parts.append(node.id)
        return parts[::-1]


# -------------------------------------------------------------------- parser
class Parser:
    """``Parser(func, name, mode, self_type).result`` is the function's
    ``ir.Definition``; ``includes`` lists the headers its ``import``s name."""

    def __init__(self, func, name: str, mode: str, self_type: BaseType | None) -> None:
        self.logger = Logger(self)
        self.func, self.name, self.mode, self.self_type = func, name, mode, self_type
        self.source = _Source.of(func)
        self.file = self.source.file
        self.names = _Lookup(func)
        self.scope = Scope(regions=[mode])
        self.return_type: BaseType | None = None
        self.statement_rules = {
            ast.Return: self.s_return, ast.Pass: lambda n: [], ast.Break: self.s_break,
            ast.Continue: self.s_continue, ast.If: self.s_if, ast.While: self.s_while,
            ast.Expr: self.s_expr, ast.With: self.s_with, ast.Assign: self.s_assign,
            ast.AugAssign: self.s_augassign, ast.For: self.s_for, ast.Import: self.s_import,
        }
        self.expression_rules = {
            ast.Constant: lambda n: self.constant(n, n.value), ast.UnaryOp: self.e_unary,
            ast.BinOp: self.e_binary, ast.BoolOp: self.e_logic, ast.Compare: self.e_compare,
            ast.IfExp: self.e_select, ast.Name: self.e_named, ast.Attribute: self.e_named,
            ast.Subscript: self.e_subscript, ast.Call: self.e_call,
        }
        self.ir = self.definition(self.source.tree)

    @property
    def result(self) -> ir.Definition:
        return self.ir

    @property
    def includes(self) -> list:
        return self.scope.includes

    # ------------------------------------------------------------- reporting
    def fail(self, node, message: str) -> NoReturn:
        self.logger.dead(f"File {self.file}, line {getattr(node, 'lineno', 1) - 1}, in {self.name}",
                         f"  Syntax error: {message}")

    def unsupported(self, node) -> NoReturn:
        self.fail(node, f"Python syntax '{type(node).__name__}' is currently unsupported")

    def at(self, node) -> ir.Location:
        return ir.Location(self.file, self.name, getattr(node, "lineno", 1) - 1)

    # ------------------------------------------------------------- definition
    def definition(self, tree: ast.FunctionDef) -> ir.Definition:
        params = []
        for arg_name, p in inspect.signature(self.func).parameters.items():
            if p.kind != inspect.Parameter.POSITIONAL_OR_KEYWORD:
                self.fail(tree, f"Argument '{arg_name}' of kind '{p.kind}' is not supported")
            annotated = p.annotation is not inspect.Parameter.empty
            if not annotated and self.self_type is None:
                self.fail(tree, f"Argument '{arg_name}' requires type annotation")
            t = parse_annotation(p.annotation, self.names.table) if annotated else self.self_type
            if t is None or isinstance(t, Void):
                self.fail(tree, f"Argument '{arg_name}' requires non-void type annotation ({p.annotation})")
            self.scope.symbols[arg_name] = ir.Variable(arg_name, t)
            params.append((arg_name, t))
        ret = inspect.signature(self.func).return_annotation
        self.return_type = None if ret is inspect.Signature.empty else parse_annotation(ret, self.names.table)
        if self.return_type is None or isinstance(self.return_type, Reference):
            self.fail(tree, f"Invalid return type '{self.return_type}'")
        body = tree.body
        if body and isinstance(body[0], ast.Expr) and isinstance(body[0].value, ast.Constant) \
                and isinstance(body[0].value.value, str):
            body = body[1:]  # a docstring documents the kernel, it is not code
        stmts = [] if self.mode == "external" else self.block(body)
        return ir.Definition(self.at(tree), self.name, self.mode, ir.Signature(params, self.return_type),
                             self.scope.symbols, stmts)

    # ------------------------------------------------------------- statements
    def block(self, nodes, region: str | None = None) -> list:
        if region is not None:
            self.scope.regions.append(region)
        out = []
        for node in nodes:
            rule = self.statement_rules.get(type(node))
            if rule is None:
                self.unsupported(node)
            out.extend(rule(node))
        if region is not None:
            self.scope.regions.pop()
        return out

    def s_return(self, node: ast.Return) -> list:
        value = None if node.value is None else self.expression(node.value)
        if value is not None and value.type != self.return_type:
            self.fail(node, f"Incompatible return type '{value.type}' with '{self.return_type}'")
        return [ir.Return(self.at(node), value)]

    def s_break(self, node) -> list:
        return [ir.Break(self.at(node))]

    def s_continue(self, node) -> list:
        return [ir.Continue(self.at(node))]

    def s_if(self, node: ast.If) -> list:
        condition = self.expression(node.test)
        self.scope.regions.append("if")
        then, orelse = self.block(node.body), self.block(node.orelse)
        self.scope.regions.pop()
        return [ir.If(self.at(node), condition, then, orelse)]

    def s_while(self, node: ast.While) -> list:
        condition = self.expression(node.test)
        if node.orelse:
            self.fail(node, "While statement does not support else clause")
        return [ir.While(self.at(node), condition, self.block(node.body, "while"))]

    def s_expr(self, node: ast.Expr) -> list:
        if self.scope.region != "c":
            return [ir.Evaluation(self.at(node), self.expression(node.value))]
        text = node.value.value if isinstance(node.value, ast.Constant) else None
        return [ir.Inline(self.at(node), text)] if isinstance(text, str) else []

    def s_with(self, node: ast.With) -> list:
        if len(node.items) != 1:
            self.fail(node, "Only one pragma switch at once")
        pragma = node.items[0].context_expr
        if not isinstance(pragma, ast.Call):
            self.fail(node, f"Invalid pragma switch '{pragma}'")
        from . import lang
        which = self.global_value(pragma.func)
        if which is lang.c:
            return self.block(node.body, "c")
        if which is lang.boundary:
            mask = int_literal(pragma.args[0]) if len(pragma.args) == 1 else None
            if mask is None or not isinstance(pragma.args[0], ast.Constant):
                self.fail(node, "Invalid pragram switch 'boundary")
            self.scope.mask = mask
            body = self.block(node.body)
            self.scope.mask = 0
            return body
        self.fail(node, f"Unknown pragma switch '{which}'")

    def s_assign(self, node: ast.Assign) -> list:
        value = self.expression(node.value)
        if isinstance(value.type, GridType):
            self.fail(node, "Incompatible assignment to grid type")
        if len(node.targets) != 1:
            self.fail(node, "Multiple assignment is not supported")
        target = node.targets[0]
        terminal = self.terminal(target)
        if terminal is None:
            if not isinstance(target, ast.Name):
                self.fail(node, f"Undefined identifier {terminal}")
            var = self.scope.symbols[target.id] = ir.Variable(target.id, value.type)
            terminal = ir.Identifier(self.at(node), value.type, "load", var)
        if terminal.type != value.type:
            self.fail(node, f"Incompatible assignment from type {value.type} to {terminal.type}")
        return [ir.Assignment(self.at(node), terminal, value)]

    def s_augassign(self, node: ast.AugAssign) -> list:
        value = self.expression(node.value)
        target = self.terminal(node.target)
        if target is None:
            self.fail(node, f"Undefined identifier {target}")
        if isinstance(target, ir.Stencil):
            # a store inside the right-hand side makes the reference's stencil
            # classifier assert (xgrid/lang/generator.py:57-59); report it instead
            self.fail(node, "Augmented assignment to a grid is not supported, write g[..] = g[..][0] op x")
        op = ARITH_OPS.get(type(node.op))
        if op is None:
            self.fail(node, f"Unsupported binary operator '{type(node.op).__name__}'")
        if arithmetic_type(op, target.type, value.type) is None:
            self.fail(node, f"Incompatible binary operator '{op.value}' with type '{target.type}' and '{value.type}'")
        rtype = target.type
        if op is ir.BinaryOperator.Pow:  # the augmented form ignores the configured precision
            wide = isinstance(target.type, Floating) and value.type.width_bits == 64
            rtype = Floating(DOUBLE if wide else 4)
        loc = self.at(node)
        current = ir.Identifier(loc, target.type, "load", target.variable) if isinstance(target, ir.Identifier) \
            else target
        return [ir.Assignment(loc, target, ir.Binary(loc, rtype, current, value, op))]

    def s_for(self, node: ast.For) -> list:
        if not isinstance(node.target, ast.Name):
            self.fail(node, "For loop variable should be a name")
        rng = node.iter
        if not (isinstance(rng, ast.Call) and isinstance(rng.func, ast.Name) and rng.func.id == "range"):
            self.fail(node, "For loop only supports range")
        if len(rng.args) not in (2, 3):
            self.fail(node, "For loop requires start:end:step or start:end")
        start, end, *step = (self.expression(a) for a in rng.args)
        step = step[0] if step else ir.Constant(self.at(node), Integer(INT), 1)
        for bound in (start, end, step):
            if bound.type != step.type or not isinstance(bound.type, Number):
                self.fail(node, f"Incompatible loop range type '{bound.type}'")
        var = self.scope.symbols.setdefault(node.target.id, ir.Variable(node.target.id, step.type))
        if var.type != step.type:
            self.fail(node, f"Incompatible loop variable type '{var.type}' with range type '{step.type}'")
        return [ir.For(self.at(node), var, start, end, step, self.block(node.body))]

    def s_import(self, node: ast.Import) -> list:
        for alias in node.names:
            if alias.asname is not None:
                self.fail(node, f"Using import as include requires no alias for '{alias.name}'")
            self.scope.includes.append(alias.name.replace(".", "/") + ".h")
        return []

    # ------------------------------------------------------------ expressions
    def expression(self, node) -> ir.Expression:
        rule = self.expression_rules.get(type(node))
        if rule is None:
            self.unsupported(node)
        return rule(node)

    def constant(self, node, value) -> ir.Constant:
        t = literal_type(value)
        if t is None:
            self.fail(node, f"Incompatible constant '{value}' of type '{type(value)}'")
        return ir.Constant(self.at(node), t, value)

    def e_unary(self, node: ast.UnaryOp) -> ir.Expression:
        op = UNARY_OPS.get(type(node.op))
        if op is None:
            self.fail(node, f"Unsupported unary operator '{type(node.op).__name__}'")
        operand = self.expression(node.operand)
        if not unary_accepts(op, operand.type):
            self.fail(node, f"Incompatible unary operator '{op.value}' with type '{operand.type}'")
        return ir.Unary(self.at(node), operand.type, operand, op)

    def e_binary(self, node: ast.BinOp) -> ir.Expression:
        op = ARITH_OPS.get(type(node.op))
        if op is None:
            self.fail(node, f"Unsupported binary operator '{type(node.op).__name__}'")
        left, right = self.expression(node.left), self.expression(node.right)
        rtype = arithmetic_type(op, left.type, right.type)
        if rtype is None:
            self.fail(node, f"Incompatible binary operator '{op.value}' with type '{left.type}' and '{right.type}'")
        return ir.Binary(self.at(node), rtype, left, right, op)

    def e_logic(self, node: ast.BoolOp) -> ir.Expression:
        loc, op = self.at(node), LOGIC_OPS[type(node.op)]
        operands = [self.expression(part) for part in node.values]
        acc = None
        for operand in operands:
            if not isinstance(operand.type, Boolean):
                self.fail(node, f"Incompatible boolean operator '{op.value}' with '{operand.type}'")
            acc = operand if acc is None else ir.Binary(loc, Boolean(), acc, operand, op)
        return acc

    def e_compare(self, node: ast.Compare) -> ir.Expression:
        loc = self.at(node)
        first = self.expression(node.left)
        if not isinstance(first.type, Number):
            self.fail(node, f"Incompatible compare expression with type '{first.type}'")
        others = [self.expression(c) for c in node.comparators]
        acc = None
        for py_op, other in zip(node.ops, others):
            op = COMPARE_OPS[type(py_op)]
            if other.type != first.type:
                self.fail(node, f"Incompatible compare operator '{op.value}' with type '{first.type}' and "
                                f"'{other.type}'")
        for py_op, other in zip(node.ops, others):
            # ``a < b < c`` compares ``a`` with ``b`` and ``a`` with ``c`` (the reference's reading)
            term = ir.Binary(loc, Boolean(), first, other, COMPARE_OPS[type(py_op)])
            acc = term if acc is None else ir.Binary(loc, Boolean(), acc, term, ir.BinaryOperator.And)
        return acc

    def e_select(self, node: ast.IfExp) -> ir.Expression:
        condition = self.expression(node.test)
        if not isinstance(condition.type, Boolean):
            self.fail(node, f"Incompatible condition type '{condition.type}' of if expression")
        a, b = self.expression(node.body), self.expression(node.orelse)
        if a.type != b.type or not isinstance(a.type, Value):
            self.fail(node, f"Incompatible type '{a.type}' and '{b.type}' of if expression")
        return ir.Condition(self.at(node), a.type, condition, a, b)

    def e_named(self, node) -> ir.Expression:
        local = self.terminal(node)
        return local if local is not None else self.constant(node, self.global_value(node))

    def e_subscript(self, node: ast.Subscript) -> ir.Expression:
        return self.terminal(node)

    # ------------------------------------------------------ names and access
    def global_value(self, node):
        parts = self.names.chain(node)
        if parts is None:
            bad = node
            while isinstance(bad, ast.Attribute):
                bad = bad.value
            self.unsupported(bad)
        value, seen = self.names.table, ["globals"]
        for part in parts:
            try:
                value = value[part] if isinstance(value, dict) else getattr(value, part)
            except (KeyError, AttributeError):
                self.fail(node, f"Undefined attribute '{part}' of '{'.'.join(seen)}'")
            seen.append(part)
        return value

    def terminal(self, node) -> ir.Terminal | None:
        """The storage location ``node`` names inside the body: a stencil access,
        a struct field of a local, a local; None when it names something global."""
        if isinstance(node, ast.Name):
            var = self.scope.symbols.get(node.id)
            if var is None:
                return None
            vtype = var.type.element if isinstance(var.type, Pointer) else var.type
            return ir.Identifier(self.at(node), vtype, ctx_of(node.ctx), var)
        if isinstance(node, ast.Attribute):
            owner = self.terminal(node.value)
            if owner is None or not isinstance(owner.type, Structure) or node.attr not in owner.type.elements_map:
                return None
            return ir.Access(self.at(node), owner.type.elements_map[node.attr], ctx_of(node.ctx), owner, node.attr)
        if isinstance(node, ast.Subscript):
            return self.stencil(node)
        self.unsupported(node)

    def stencil(self, node: ast.Subscript) -> ir.Stencil:
        """``g[offsets]`` or ``g[offsets][t]``."""
        if isinstance(node.value, ast.Subscript):
            time = int_literal(node.slice)
            if time is None:
                self.fail(node.value, f"Invalid time dimension subscript to '{type(node.value).__name__}")
            access = node.value
        else:
            time = 0 if ctx_of(node.ctx) == "store" else -1
            access = node
        if not isinstance(access.value, ast.Name):
            self.fail(access, f"Incompatible subscript to '{type(access.value).__name__}' under context "
                              f"'{self.scope.region}'")
        var = self.scope.symbols.get(access.value.id)
        if var is None:
            self.fail(access, f"Undefined identifier '{access.value.id}'")
        if not isinstance(var.type, GridType):
            self.fail(access, f"Incompatible subscript to type '{var.type}'")
        items = access.slice.elts if isinstance(access.slice, ast.Tuple) else [access.slice]
        offsets = []
        for item in items:
            off = int_literal(item)
            if off is None:
                self.fail(access, f"Incompatible subscript '{ast.unparse(item)}'")
            offsets.append(off)
        if len(offsets) != var.type.dimension:
            self.fail(access, f"Incompatible subscript length '{len(offsets)}' with dimension {var.type.dimension}")
        return ir.Stencil(self.at(access), var.type.element, ctx_of(access.ctx), var, time, tuple(offsets),
                          self.scope.mask)

    # ------------------------------------------------------------------ calls
    def e_call(self, node: ast.Call) -> ir.Expression:
        from .operator import Operator
        receiver = self.terminal(node.func.value) if isinstance(node.func, ast.Attribute) else None
        if receiver is not None:  # method call on a struct value
            if not isinstance(receiver.type, Structure):
                self.fail(node, f"Invalid method call on type {receiver.type}")
            target = getattr(receiver.type.dataclass, node.func.attr, None)
            label = f"{receiver.type.dataclass.__qualname__}.{node.func.attr}"
            args = [receiver]
        else:
            target, label, args = self.global_value(node.func), None, []
        if target is typing.cast:
            if len(node.args) != 2:
                self.fail(node, f"Cast requires 2 arguments, got {len(node.args)}")
            to = parse_annotation(self.global_value(node.args[0]), self.names.table)
            if to is None:
                self.fail(node, "Invalid cast type")
            return ir.Cast(self.at(node), to, self.expression(node.args[1]))
        args += [self.expression(a) for a in node.args]
        if isinstance(target, type):  # a dataclass builds a struct value
            stype = parse_annotation(target, self.names.table)
            if not isinstance(stype, Structure):
                self.fail(node, f"Invalid type constructor '{target.__name__}'")
            target = ir.Constructor(stype, ir.Signature(list(stype.elements), stype), f"{stype.name}.constructor")
            label = target.name
        if not isinstance(target, (Operator, ir.Constructor)):
            lazy = getattr(target, "__xgrid_method", None)
            if lazy is None or receiver is None:
                self.fail(node, f"Invalid call to object '{target}', it is not an operator")
            target = Operator(target, "function", lazy[0], lazy[1], receiver.type)
        label = label or target.name
        params = target.signature.arguments
        if len(params) != len(args):
            self.fail(node, f"Operator '{label}' requires {len(params)} arguments, but got {len(args)}")
        if isinstance(target, Operator) and target.mode == "external" and target.typecheck_override is not None:
            try:
                rtype = target.typecheck_override([a.type for a in args])
            except Exception as e:  # noqa: BLE001 - the override's message becomes the error
                self.fail(node, e.args[0])
            if target.name in ("shape", "dimension"):
                if not isinstance(args[0], ir.Identifier):
                    self.fail(node, f"Incompatible '{target.name}' to argument '{args[0]}'")
                return ir.GridInfo(self.at(node), Integer(INT), target.name, args[0].variable,
                                   args[1] if target.name == "shape" else None)
            return ir.Call(self.at(node), rtype, target, args)
        for (pname, ptype), a in zip(params, args):
            if ptype != a.type:
                self.fail(node, f"Incompatible type '{a.type}' with '{ptype}' of argument '{pname}, operator "
                                f"'{label}'")
        return ir.Call(self.at(node), target.signature.return_type, target, args)
