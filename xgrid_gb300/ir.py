"""Typed IR produced by the parser and consumed by the CUDA generator and the oracle.

Node set and meaning follow xgrid/lang/ir/{statement,expression}.py: statements
``Definition, Return, Break, Continue, If, While, Evaluation, Assignment, Inline,
For``; expressions ``Binary, Unary, Condition, Constant, Cast, Identifier, Stencil,
Access, Call, GridInfo``.  A ``Stencil`` is one read or write of a grid at a
relative space offset and a time offset (0 = the level being written, -1 = the
previous level, ...) under the ``with boundary(k)`` mask that was active when it
was parsed.
"""
from __future__ import annotations

import dataclasses
import enum
from typing import Any, Literal, Optional

from .types import BaseType


@dataclasses.dataclass
class Location:
    file: str
    func: str
    line: int

    def __repr__(self) -> str:
        return f"File {self.file}, line {self.line}, at {self.func}"


@dataclasses.dataclass(eq=False)
class Variable:
    name: str
    type: BaseType


@dataclasses.dataclass(eq=False)
class Node:
    location: Location


# ------------------------------------------------------------------ expressions
class BinaryOperator(enum.Enum):
    Add = "+"
    Sub = "-"
    Mul = "*"
    Div = "/"
    Pow = "^"
    Mod = "%"
    Eq = "=="
    Gt = ">"
    Ge = ">="
    Lt = "<"
    Le = "<="
    Neq = "!="
    And = "&&"
    Or = "||"

    def is_compare(self) -> bool:
        return self in (BinaryOperator.Eq, BinaryOperator.Gt, BinaryOperator.Ge,
                        BinaryOperator.Lt, BinaryOperator.Le, BinaryOperator.Neq)

    def is_logic(self) -> bool:
        return self in (BinaryOperator.And, BinaryOperator.Or)


class UnaryOperator(enum.Enum):
    Pos = "+"
    Neg = "-"
    Not = "!"


@dataclasses.dataclass(eq=False)
class Expression(Node):
    type: BaseType


@dataclasses.dataclass(eq=False)
class Binary(Expression):
    left: Expression
    right: Expression
    operator: BinaryOperator


@dataclasses.dataclass(eq=False)
class Unary(Expression):
    right: Expression
    operator: UnaryOperator


@dataclasses.dataclass(eq=False)
class Condition(Expression):
    condition: Expression
    body: Expression
    orelse: Expression


@dataclasses.dataclass(eq=False)
class Constant(Expression):
    value: Any


@dataclasses.dataclass(eq=False)
class Cast(Expression):
    value: Expression


@dataclasses.dataclass(eq=False)
class Terminal(Expression):
    context: Literal["load", "store"]


@dataclasses.dataclass(eq=False)
class Identifier(Terminal):
    variable: Variable


@dataclasses.dataclass(eq=False)
class Stencil(Terminal):
    variable: Variable
    time_offset: int
    space_offset: tuple
    boundary_mask: int = 0


@dataclasses.dataclass(eq=False)
class Access(Terminal):
    value: Terminal
    attribute: str


@dataclasses.dataclass
class Signature:
    arguments: list
    return_type: BaseType

    def __post_init__(self):
        self.argnames_map = dict(self.arguments)


@dataclasses.dataclass(eq=False)
class Constructor:
    """A dataclass used as a call target: builds a struct value."""

    type: BaseType
    signature: Signature
    name: str = ""


@dataclasses.dataclass(eq=False)
class Call(Expression):
    operator: Any  # Operator | Constructor
    arguments: list


@dataclasses.dataclass(eq=False)
class GridInfo(Expression):
    info: Literal["shape", "dimension"]
    variable: Variable
    dimension: Optional[Expression]


# ------------------------------------------------------------------- statements
@dataclasses.dataclass(eq=False)
class Statement(Node):
    pass


@dataclasses.dataclass(eq=False)
class Definition(Statement):
    name: str
    mode: str
    signature: Signature
    scope: dict
    body: list


@dataclasses.dataclass(eq=False)
class Return(Statement):
    value: Optional[Expression]


@dataclasses.dataclass(eq=False)
class Break(Statement):
    pass


@dataclasses.dataclass(eq=False)
class Continue(Statement):
    pass


@dataclasses.dataclass(eq=False)
class If(Statement):
    condition: Expression
    body: list
    orelse: list


@dataclasses.dataclass(eq=False)
class While(Statement):
    condition: Expression
    body: list


@dataclasses.dataclass(eq=False)
class Evaluation(Statement):
    value: Expression


@dataclasses.dataclass(eq=False)
class Assignment(Statement):
    terminal: Terminal
    value: Expression


@dataclasses.dataclass(eq=False)
class Inline(Statement):
    source: str


@dataclasses.dataclass(eq=False)
class For(Statement):
    variable: Variable
    start: Expression
    end: Expression
    step: Expression
    body: list


def walk(node):
    """Yield every IR node below ``node`` (pre-order), including ``node``."""
    if isinstance(node, list):
        for item in node:
            yield from walk(item)
        return
    if not isinstance(node, Node):
        return
    yield node
    for field in dataclasses.fields(node):
        if field.name in ("location", "type", "variable", "operator", "scope", "signature"):
            continue
        value = getattr(node, field.name)
        if isinstance(value, (Node, list)):
            yield from walk(value)


def stencils(expr) -> list:
    return [n for n in walk(expr) if isinstance(n, Stencil)]
