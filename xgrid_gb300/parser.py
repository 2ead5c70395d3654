"""Python source → typed IR for ``@xgrid.kernel`` / ``@xgrid.function`` bodies.

The accepted syntax, the typing rules and the error messages follow the
reference parser (xgrid/lang/parser.py:54-641):

* subscripts ``g[o0, ..., oN-1]`` are stencil accesses with integer-literal
  offsets (parser.py:456-510); a load without a time subscript reads time -1, a
  store writes time 0, ``g[...][t]`` names time ``t`` explicitly (parser.py:512-523);
* ``with xgrid.boundary(k):`` sets the mask of the stencils parsed inside it and
  ``with xgrid.c():`` turns string statements into inline source
  (parser.py:208-235);
* binary operators require both operands of the same numeric type; ``**`` yields
  FP64 when the left operand is FP64 and ``float`` otherwise (parser.py:365-384);
* comparisons chain with ``&&`` (parser.py:396-414); globals fold to constants
  (parser.py:548-554); calls resolve operators, dataclass constructors, methods,
  ``typing.cast`` and the built-in ``shape``/``dimension`` (parser.py:559-641).

Every error goes through ``Logger.dead`` and is raised as ``Exception``.
"""
from __future__ import annotations

import ast
import functools
import inspect
import struct
import textwrap
import typing
from typing import NoReturn, cast as typing_cast

from . import ir
from .config import get_config
from .log import Logger
from .types import (BaseType, Boolean, Floating, GridType, Integer, Number, Pointer,
                    Reference, Structure, Value, Void, parse_annotation)

_UNARY = {ast.UAdd: ir.UnaryOperator.Pos, ast.USub: ir.UnaryOperator.Neg,
          ast.Not: ir.UnaryOperator.Not}
_BINARY = {ast.Add: ir.BinaryOperator.Add, ast.Sub: ir.BinaryOperator.Sub,
           ast.Mult: ir.BinaryOperator.Mul, ast.Div: ir.BinaryOperator.Div,
           ast.Pow: ir.BinaryOperator.Pow, ast.Mod: ir.BinaryOperator.Mod,
           ast.Eq: ir.BinaryOperator.Eq, ast.NotEq: ir.BinaryOperator.Neq,
           ast.Gt: ir.BinaryOperator.Gt, ast.GtE: ir.BinaryOperator.Ge,
           ast.Lt: ir.BinaryOperator.Lt, ast.LtE: ir.BinaryOperator.Le,
           ast.And: ir.BinaryOperator.And, ast.Or: ir.BinaryOperator.Or}


def _ctx(node) -> str:
    return "load" if isinstance(node, ast.Load) else "store"


def _int_literal(node) -> int | None:
    """Value of ``k`` or ``-k`` for an int literal ``k``, else None."""
    if isinstance(node, ast.Constant) and type(node.value) is int:
        return node.value
    if (isinstance(node, ast.UnaryOp) and isinstance(node.op, ast.USub)
            and isinstance(node.operand, ast.Constant) and type(node.operand.value) is int):
        return -node.operand.value
    return None


class Parser:
    def __init__(self, func, name: str, mode: str, self_type: BaseType | None) -> None:
        self.logger = Logger(self)
        self.func = func
        self.name = name
        self.mode = mode
        self.self_type = self_type
        self.file = inspect.getsourcefile(func) or "<unknown>"
        lines, lineno = inspect.getsourcelines(func)
        source = textwrap.dedent("".join(lines))
        tree = ast.parse(source, self.file).body[0]
        ast.increment_lineno(tree, lineno)
        self.context_stack = [mode]
        self.scope: dict[str, ir.Variable] = {}
        self.boundary_mask = 0
        self.args: list = []
        self.global_scope = dict(func.__globals__)
        self.global_scope.update({"int": int, "float": float, "bool": bool})
        try:  # constants captured from an enclosing function fold like globals
            self.global_scope.update(inspect.getclosurevars(func).nonlocals)
        except (TypeError, ValueError):
            pass
        self.includes: list[str] = []
        self.ir = self.visit(tree)

    @property
    def result(self) -> ir.Definition:
        return self.ir

    @property
    def context(self) -> str:
        return self.context_stack[-1]

    def syntax_error(self, node, message: str) -> NoReturn:
        self.logger.dead(f"File {self.file}, line {getattr(node, 'lineno', 1) - 1}, in {self.name}",
                         f"  Syntax error: {message}")

    def location(self, node) -> ir.Location:
        return ir.Location(self.file, self.name, getattr(node, "lineno", 1) - 1)

    def visit(self, node):
        method = getattr(self, "visit_" + type(node).__name__, None)
        if method is None:
            self.syntax_error(node, f"Python syntax '{type(node).__name__}' is currently unsupported")
        return method(node)

    def visits(self, nodes) -> list:
        out = []
        for node in nodes:
            item = self.visit(node)
            if isinstance(item, list):
                out.extend(item)
            elif item is not None:
                out.append(item)
        return out

    # ------------------------------------------------------------- definition
    def visit_FunctionDef(self, node: ast.FunctionDef):
        sig = inspect.signature(self.func)
        for arg_name, param in sig.parameters.items():
            if param.kind != inspect.Parameter.POSITIONAL_OR_KEYWORD:
                self.syntax_error(node, f"Argument '{arg_name}' of kind '{param.kind}' is not supported")
            if param.annotation is inspect.Parameter.empty and self.self_type is None:
                self.syntax_error(node, f"Argument '{arg_name}' requires type annotation")
            if param.annotation is inspect.Parameter.empty:
                arg_type = self.self_type
            else:
                arg_type = parse_annotation(param.annotation, self.global_scope)
            if arg_type is None or isinstance(arg_type, Void):
                self.syntax_error(node, f"Argument '{arg_name}' requires non-void type annotation ({param.annotation})")
            self.scope[arg_name] = ir.Variable(arg_name, arg_type)
            self.args.append((arg_name, arg_type))
        ret = sig.return_annotation
        ret_type = None if ret is inspect.Signature.empty else parse_annotation(ret, self.global_scope)
        if ret_type is None or isinstance(ret_type, Reference):
            self.syntax_error(node, f"Invalid return type '{ret_type}'")
        self.return_type = ret_type
        stmts = node.body
        if stmts and isinstance(stmts[0], ast.Expr) and isinstance(stmts[0].value, ast.Constant) \
                and isinstance(stmts[0].value.value, str):
            stmts = stmts[1:]  # a leading docstring documents the kernel; it is not code
        body = [] if self.mode == "external" else self.visits(stmts)
        return ir.Definition(self.location(node), self.name, self.mode,
                             ir.Signature(self.args, self.return_type), self.scope, body)

    # ------------------------------------------------------------- statements
    def visit_Return(self, node: ast.Return):
        value = None if node.value is None else self.visit(node.value)
        if value is not None and value.type != self.return_type:
            self.syntax_error(node, f"Incompatible return type '{value.type}' with '{self.return_type}'")
        return ir.Return(self.location(node), value)

    def visit_Pass(self, node):
        return []

    def visit_Break(self, node):
        return ir.Break(self.location(node))

    def visit_Continue(self, node):
        return ir.Continue(self.location(node))

    def visit_If(self, node: ast.If):
        condition = self.visit(node.test)
        self.context_stack.append("if")
        body = self.visits(node.body)
        orelse = self.visits(node.orelse)
        self.context_stack.pop()
        return ir.If(self.location(node), condition, body, orelse)

    def visit_While(self, node: ast.While):
        condition = self.visit(node.test)
        if node.orelse:
            self.syntax_error(node, "While statement does not support else clause")
        self.context_stack.append("while")
        body = self.visits(node.body)
        self.context_stack.pop()
        return ir.While(self.location(node), condition, body)

    def visit_Expr(self, node: ast.Expr):
        if self.context == "c":
            if isinstance(node.value, ast.Constant) and isinstance(node.value.value, str):
                return ir.Inline(self.location(node), node.value.value)
            return None
        return ir.Evaluation(self.location(node), self.visit(node.value))

    def visit_With(self, node: ast.With):
        if len(node.items) != 1:
            self.syntax_error(node, "Only one pragma switch at once")
        item = node.items[0].context_expr
        if not isinstance(item, ast.Call):
            self.syntax_error(node, f"Invalid pragma switch '{item}'")
        target = self.resolve_global(item.func)
        from . import lang
        if target is lang.c:
            self.context_stack.append("c")
            body = self.visits(node.body)
            self.context_stack.pop()
            return body
        if target is lang.boundary:
            args = item.args
            if len(args) != 1 or not isinstance(args[0], ast.Constant) or type(args[0].value) is not int:
                self.syntax_error(node, "Invalid pragram switch 'boundary")
            self.boundary_mask = args[0].value
            body = self.visits(node.body)
            self.boundary_mask = 0
            return body
        self.syntax_error(node, f"Unknown pragma switch '{target}'")

    def visit_Assign(self, node: ast.Assign):
        location = self.location(node)
        value = self.visit(node.value)
        if isinstance(value.type, GridType):
            self.syntax_error(node, "Incompatible assignment to grid type")
        if len(node.targets) != 1:
            self.syntax_error(node, "Multiple assignment is not supported")
        target = node.targets[0]
        terminal = self.resolve_local(target)
        if terminal is None:
            if not isinstance(target, ast.Name):
                self.syntax_error(node, f"Undefined identifier {terminal}")
            variable = ir.Variable(target.id, value.type)
            self.scope[target.id] = variable
            terminal = ir.Identifier(location, value.type, "load", variable)
        if terminal.type != value.type:
            self.syntax_error(node, f"Incompatible assignment from type {value.type} to {terminal.type}")
        return ir.Assignment(location, terminal, value)

    def visit_AugAssign(self, node: ast.AugAssign):
        value = self.visit(node.value)
        target = self.resolve_local(node.target)
        if target is None:
            self.syntax_error(node, f"Undefined identifier {target}")
        if isinstance(target, ir.Stencil):
            # the reference's stencil classifier asserts on a store inside the
            # right-hand side (xgrid/lang/generator.py:57-59); report it instead.
            self.syntax_error(node, "Augmented assignment to a grid is not supported, write g[..] = g[..][0] op x")
        op_type = type(node.op)
        if op_type not in _BINARY:
            self.syntax_error(node, f"Unsupported binary operator '{op_type.__name__}'")
        op = _BINARY[op_type]
        if not isinstance(target.type, Number) or not isinstance(value.type, Number) or target.type != value.type:
            self.syntax_error(node, f"Incompatible binary operator '{op.value}' with type '{target.type}' and '{value.type}'")
        if op is ir.BinaryOperator.Pow:
            rtype = Floating(8) if isinstance(target.type, Floating) and value.type.width_bits == 64 else Floating(4)
        else:
            rtype = target.type
        loc = self.location(node)
        load = ir.Identifier(loc, target.type, "load", target.variable) if isinstance(target, ir.Identifier) else target
        return ir.Assignment(loc, target, ir.Binary(loc, rtype, load, value, op))

    def visit_For(self, node: ast.For):
        if not isinstance(node.target, ast.Name):
            self.syntax_error(node, "For loop variable should be a name")
        it = node.iter
        if not (isinstance(it, ast.Call) and isinstance(it.func, ast.Name) and it.func.id == "range"):
            self.syntax_error(node, "For loop only supports range")
        if len(it.args) not in (2, 3):
            self.syntax_error(node, "For loop requires start:end:step or start:end")
        bounds = [self.visit(a) for a in it.args]
        if len(bounds) == 2:
            bounds.append(ir.Constant(self.location(node), Integer(struct.calcsize("i")), 1))
        rtype = bounds[2].type
        for b in bounds:
            if b.type != rtype or not isinstance(b.type, Number):
                self.syntax_error(node, f"Incompatible loop range type '{b.type}'")
        var_id = node.target.id
        if var_id not in self.scope:
            self.scope[var_id] = ir.Variable(var_id, rtype)
        var = self.scope[var_id]
        if var.type != rtype:
            self.syntax_error(node, f"Incompatible loop variable type '{var.type}' with range type '{rtype}'")
        body = self.visits(node.body)
        return ir.For(self.location(node), var, bounds[0], bounds[1], bounds[2], body)

    def visit_Import(self, node: ast.Import):
        for alias in node.names:
            if alias.asname is not None:
                self.syntax_error(node, f"Using import as include requires no alias for '{alias.name}'")
            self.includes.append(alias.name.replace(".", "/") + ".h")
        return []

    # ------------------------------------------------------------ expressions
    def parse_constant(self, node, value) -> ir.Constant:
        types = {int: Integer(struct.calcsize("i")), float: Floating(get_config().fsize), bool: Boolean()}
        if type(value) not in types:
            self.syntax_error(node, f"Incompatible constant '{value}' of type '{type(value)}'")
        return ir.Constant(self.location(node), types[type(value)], value)

    def visit_Constant(self, node: ast.Constant):
        return self.parse_constant(node, node.value)

    def visit_UnaryOp(self, node: ast.UnaryOp):
        op_type = type(node.op)
        if op_type not in _UNARY:
            self.syntax_error(node, f"Unsupported unary operator '{op_type.__name__}'")
        op = _UNARY[op_type]
        right = self.visit(node.operand)
        if (op is ir.UnaryOperator.Not and not isinstance(right.type, Boolean)) or \
                (op in (ir.UnaryOperator.Pos, ir.UnaryOperator.Neg) and not isinstance(right.type, Number)):
            self.syntax_error(node, f"Incompatible unary operator '{op.value}' with type '{right.type}'")
        return ir.Unary(self.location(node), right.type, right, op)

    def visit_BinOp(self, node: ast.BinOp):
        op_type = type(node.op)
        if op_type not in _BINARY:
            self.syntax_error(node, f"Unsupported binary operator '{op_type.__name__}'")
        op = _BINARY[op_type]
        left = self.visit(node.left)
        right = self.visit(node.right)
        if not isinstance(left.type, Number) or not isinstance(right.type, Number) or left.type != right.type:
            self.syntax_error(node, f"Incompatible binary operator '{op.value}' with type '{left.type}' and '{right.type}'")
        if op is ir.BinaryOperator.Pow:
            if isinstance(left.type, Floating) and left.type.width_bits == 64:
                rtype = Floating(struct.calcsize("d"))
            else:
                rtype = Floating(get_config().fsize)
        else:
            rtype = left.type
        return ir.Binary(self.location(node), rtype, left, right, op)

    def visit_BoolOp(self, node: ast.BoolOp):
        loc = self.location(node)
        op = _BINARY[type(node.op)]
        values = [self.visit(v) for v in node.values]
        for v in values:
            if not isinstance(v.type, Boolean):
                self.syntax_error(node, f"Incompatible boolean operator '{op.value}' with '{v.type}'")
        return functools.reduce(lambda a, b: ir.Binary(loc, Boolean(), a, b, op), values)

    def visit_Compare(self, node: ast.Compare):
        loc = self.location(node)
        left = self.visit(node.left)
        if not isinstance(left.type, Number):
            self.syntax_error(node, f"Incompatible compare expression with type '{left.type}'")
        comparators = [self.visit(c) for c in node.comparators]
        ops = [_BINARY[type(o)] for o in node.ops]
        for op, comp in zip(ops, comparators):
            if comp.type != left.type:
                self.syntax_error(node, f"Incompatible compare operator '{op.value}' with type '{left.type}' and '{comp.type}'")
        # every comparison in a chain takes the first operand on its left, as in the reference
        pairs = [ir.Binary(loc, Boolean(), left, comp, op) for op, comp in zip(ops, comparators)]
        return functools.reduce(lambda a, b: ir.Binary(loc, Boolean(), a, b, ir.BinaryOperator.And), pairs)

    def visit_IfExp(self, node: ast.IfExp):
        condition = self.visit(node.test)
        if not isinstance(condition.type, Boolean):
            self.syntax_error(node, f"Incompatible condition type '{condition.type}' of if expression")
        body = self.visit(node.body)
        orelse = self.visit(node.orelse)
        if body.type != orelse.type or not isinstance(body.type, Value):
            self.syntax_error(node, f"Incompatible type '{body.type}' and '{orelse.type}' of if expression")
        return ir.Condition(self.location(node), body.type, condition, body, orelse)

    def resolve_global(self, node):
        names = []
        while True:
            if isinstance(node, ast.Name):
                names.append(node.id)
                break
            if isinstance(node, ast.Attribute):
                names.append(node.attr)
                node = node.value
                continue
            self.syntax_error(node, f"Python syntax '{type(node).__name__}' is currently unsupported")
        names.reverse()
        scope = self.global_scope
        resolved = ["globals"]
        for attr in names:
            try:
                scope = scope[attr] if isinstance(scope, dict) else getattr(scope, attr)
            except (KeyError, AttributeError):
                self.syntax_error(node, f"Undefined attribute '{attr}' of '{'.'.join(resolved)}'")
            resolved.append(attr)
        return scope

    def resolve_local(self, node) -> ir.Terminal | None:
        location = self.location(node)
        if isinstance(node, ast.Subscript):
            if isinstance(node.value, ast.Subscript):
                time_offset = _int_literal(node.slice)
                if time_offset is None:
                    self.syntax_error(node.value, f"Invalid time dimension subscript to '{type(node.value).__name__}")
                grid = node.value
            else:
                time_offset = 0 if _ctx(node.ctx) == "store" else -1
                grid = node
            return self._space(grid, time_offset)
        if isinstance(node, ast.Attribute):
            value = self.resolve_local(node.value)
            if value is None or not isinstance(value.type, Structure) or node.attr not in value.type.elements_map:
                return None
            return ir.Access(location, value.type.elements_map[node.attr], _ctx(node.ctx), value, node.attr)
        if isinstance(node, ast.Name):
            variable = self.scope.get(node.id)
            if variable is None:
                return None
            vtype = variable.type.element if isinstance(variable.type, Pointer) else variable.type
            return ir.Identifier(location, vtype, _ctx(node.ctx), variable)
        self.syntax_error(node, f"Python syntax '{type(node).__name__}' is currently unsupported")

    def _space(self, grid: ast.Subscript, time_offset: int) -> ir.Stencil:
        if not isinstance(grid.value, ast.Name):
            self.syntax_error(grid, f"Incompatible subscript to '{type(grid.value).__name__}' under context '{self.context}'")
        if grid.value.id not in self.scope:
            self.syntax_error(grid, f"Undefined identifier '{grid.value.id}'")
        var = self.scope[grid.value.id]
        if not isinstance(var.type, GridType):
            self.syntax_error(grid, f"Incompatible subscript to type '{var.type}'")
        slices = grid.slice.elts if isinstance(grid.slice, ast.Tuple) else [grid.slice]
        offsets = []
        for s in slices:
            value = _int_literal(s)
            if value is None:
                self.syntax_error(grid, f"Incompatible subscript '{ast.unparse(s)}'")
            offsets.append(value)
        if len(offsets) != var.type.dimension:
            self.syntax_error(grid, f"Incompatible subscript length '{len(offsets)}' with dimension {var.type.dimension}")
        return ir.Stencil(self.location(grid), var.type.element, _ctx(grid.ctx), var, time_offset,
                          tuple(offsets), self.boundary_mask)

    def visit_Name(self, node: ast.Name):
        local = self.resolve_local(node)
        return self.parse_constant(node, self.resolve_global(node)) if local is None else local

    def visit_Attribute(self, node: ast.Attribute):
        local = self.resolve_local(node)
        return self.parse_constant(node, self.resolve_global(node)) if local is None else local

    def visit_Subscript(self, node: ast.Subscript):
        return self.resolve_local(node)

    def visit_Call(self, node: ast.Call):
        from .operator import Operator
        func_name = None
        self_type = None
        local = None
        if isinstance(node.func, ast.Attribute):
            local = self.resolve_local(node.func.value)
        if local is not None:
            if not isinstance(local.type, Structure):
                self.syntax_error(node, f"Invalid method call on type {local.type}")
            func = getattr(local.type.dataclass, node.func.attr, None)
            func_name = f"{local.type.dataclass.__qualname__}.{node.func.attr}"
            self_type = local.type
            args = [local]
        else:
            func = self.resolve_global(node.func)
            args = []

        if func is typing_cast or func is typing.cast:
            if len(node.args) != 2:
                self.syntax_error(node, f"Cast requires 2 arguments, got {len(node.args)}")
            target = parse_annotation(self.resolve_global(node.args[0]), self.global_scope)
            if target is None:
                self.syntax_error(node, "Invalid cast type")
            return ir.Cast(self.location(node), target, self.visit(node.args[1]))

        args.extend(self.visit(a) for a in node.args)

        if isinstance(func, type):
            stype = parse_annotation(func, self.global_scope)
            if stype is None or not isinstance(stype, Structure):
                self.syntax_error(node, f"Invalid type constructor '{func.__name__}'")
            func = ir.Constructor(stype, ir.Signature(list(stype.elements), stype), f"{stype.name}.constructor")
            func_name = func.name

        if not isinstance(func, (Operator, ir.Constructor)):
            flag = getattr(func, "__xgrid_method", None)
            if flag is not None and self_type is not None:
                func = Operator(func, "function", flag[0], flag[1], self_type)
            else:
                self.syntax_error(node, f"Invalid call to object '{func}', it is not an operator")

        if func_name is None:
            func_name = func.name
        expected = len(func.signature.arguments)
        if expected != len(args):
            self.syntax_error(node, f"Operator '{func_name}' requires {expected} arguments, but got {len(args)}")

        if isinstance(func, Operator) and func.mode == "external" and func.typecheck_override is not None:
            try:
                rtype = func.typecheck_override([a.type for a in args])
            except Exception as e:  # noqa: BLE001 - message forwarded as a syntax error
                self.syntax_error(node, e.args[0])
            if func.name in ("shape", "dimension"):
                if not isinstance(args[0], ir.Identifier):
                    self.syntax_error(node, f"Incompatible '{func.name}' to argument '{args[0]}'")
                return ir.GridInfo(self.location(node), Integer(struct.calcsize("i")), func.name,
                                   args[0].variable, args[1] if func.name == "shape" else None)
        else:
            for i, (arg_name, arg_type) in enumerate(func.signature.arguments):
                if arg_type != args[i].type:
                    self.syntax_error(node, f"Incompatible type '{args[i].type}' with '{arg_type}' of argument '{arg_name}, operator '{func_name}'")
            rtype = func.signature.return_type
        return ir.Call(self.location(node), rtype, func, args)
