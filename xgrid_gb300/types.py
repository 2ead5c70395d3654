"""DSL value and reference types, their ctypes layouts and the annotation parser.

The type lattice and its equality rules follow xgrid/util/typing/{__init__,value,
reference,annotation}.py: ``int`` is a 4-byte ``Integer``, ``float`` is a
``Floating`` whose width comes from ``init(precision=...)`` at parse time, ``bool``
is ``Boolean``, a dataclass becomes a by-value ``Structure``, ``ptr[T]`` a
``Pointer`` and ``grid[T, N]`` a ``GridType``.  Types compare by value, so two
annotations of the same shape are the same type.

Each type also knows its C spelling (``cname``) for the CUDA generator.
"""
from __future__ import annotations

import ctypes
import dataclasses
import struct
from typing import Any, Generic, TypeVar, get_args, get_origin


@dataclasses.dataclass
class BaseType:
    @property
    def ctype(self) -> Any:
        raise NotImplementedError

    def serialize(self, value):
        raise NotImplementedError

    def deserialize(self, value):
        return value


@dataclasses.dataclass
class Void(BaseType):
    def __repr__(self) -> str:
        return "Void"

    @property
    def cname(self) -> str:
        return "void"


@dataclasses.dataclass
class Ignore(BaseType):
    """``typing.Any``: matches every type (used by built-in externals)."""

    def __eq__(self, other):
        return True

    __hash__ = None


@dataclasses.dataclass
class Value(BaseType):
    @property
    def abbr(self) -> str:
        return ""


@dataclasses.dataclass
class Boolean(Value):
    @property
    def ctype(self):
        return ctypes.c_bool

    def serialize(self, value):
        return ctypes.c_bool(value)

    def deserialize(self, value):
        return bool(value)

    @property
    def abbr(self) -> str:
        return "b"

    @property
    def cname(self) -> str:
        return "bool"

    @property
    def nbytes(self) -> int:
        return 1

    def __repr__(self) -> str:
        return "Boolean"


@dataclasses.dataclass
class Number(Value):
    width_bytes: int

    @property
    def width_bits(self) -> int:
        return self.width_bytes * 8

    @property
    def nbytes(self) -> int:
        return self.width_bytes


_INT_CTYPES = {1: ctypes.c_int8, 2: ctypes.c_int16, 4: ctypes.c_int32, 8: ctypes.c_int64}


@dataclasses.dataclass
class Integer(Number):
    def __post_init__(self):
        if self.width_bytes not in _INT_CTYPES:
            raise ValueError(f"invalid integer width {self.width_bytes}")

    @property
    def ctype(self):
        return _INT_CTYPES[self.width_bytes]

    def serialize(self, value):
        return self.ctype(value)

    def deserialize(self, value):
        return int(value)

    @property
    def abbr(self) -> str:
        return f"i{self.width_bits}"

    @property
    def cname(self) -> str:
        return f"int{self.width_bits}_t"

    def __repr__(self) -> str:
        return f"Integer({self.width_bits})"


@dataclasses.dataclass
class Floating(Number):
    def __post_init__(self):
        if self.width_bytes not in (4, 8):
            raise ValueError(f"invalid floating width {self.width_bytes}")

    @property
    def ctype(self):
        return ctypes.c_float if self.width_bytes == 4 else ctypes.c_double

    def serialize(self, value):
        return self.ctype(value)

    def deserialize(self, value):
        return float(value)

    @property
    def abbr(self) -> str:
        return f"f{self.width_bits}"

    @property
    def cname(self) -> str:
        return "float" if self.width_bytes == 4 else "double"

    def __repr__(self) -> str:
        return f"Floating({self.width_bits})"


@dataclasses.dataclass
class Structure(Value):
    dataclass: type
    name: str
    elements: tuple

    def __post_init__(self):
        self.elements_map = dict(self.elements)
        self._ctype = type(f"st{self.name}", (ctypes.Structure,),
                           {"_fields_": [(n, t.ctype) for n, t in self.elements]})

    @property
    def ctype(self):
        return self._ctype

    def serialize(self, value):
        return self._ctype(*dataclasses.astuple(value))

    def deserialize(self, value):
        return self.dataclass(*[getattr(value, n) for n, _ in self.elements])

    @property
    def abbr(self) -> str:
        return f"st{self.name}"

    @property
    def cname(self) -> str:
        return f"struct {self.name}"

    @property
    def nbytes(self) -> int:
        return ctypes.sizeof(self._ctype)

    def __repr__(self) -> str:
        return self.name


@dataclasses.dataclass
class Reference(BaseType):
    pass


@dataclasses.dataclass
class Pointer(Reference):
    element: Value

    @property
    def ctype(self):
        return ctypes.POINTER(self.element.ctype)

    def serialize(self, value):
        return self.ctype(value)

    @property
    def cname(self) -> str:
        return f"{self.element.cname}*"

    def __repr__(self) -> str:
        return f"Pointer of {self.element!r}"


@dataclasses.dataclass
class GridType(Reference):
    """``grid[T, N]``: an N-dimensional field of T with time levels and a mask."""

    element: Value
    dimension: int

    def __repr__(self) -> str:
        return f"Grid({self.dimension}) of {self.element!r}"


# ----------------------------------------------------------------- annotations
Length = TypeVar("Length")
Elem = TypeVar("Elem")


class Annotation:
    """Marker base of the DSL annotation classes."""


class ptr(Annotation, Generic[Elem]):
    def addr(self) -> int: ...


class grid(Annotation, Generic[Elem, Length]):
    def __getitem__(self, key) -> Any: ...

    def __setitem__(self, key, value) -> Any: ...


def _fsize() -> int:
    from .config import get_config
    return get_config().fsize


def int_type() -> Integer:
    return Integer(struct.calcsize("i"))


def float_type() -> Floating:
    return Floating(_fsize())


def parse_annotation(annotation, glbs: dict | None = None) -> BaseType | None:
    """Map a Python annotation to a DSL type; ``None`` when it is not one.

    Follows xgrid/util/typing/annotation.py:31-68 (string annotations are looked up
    in ``glbs``; ``float`` width comes from the configuration).
    """
    if annotation is None:
        return Void()
    if isinstance(annotation, str):
        scope = glbs if glbs is not None else globals()
        if annotation in scope:
            annotation = scope[annotation]
        else:
            try:  # postponed annotations ("from __future__ import annotations")
                annotation = eval(annotation, dict(scope))  # noqa: S307 - user's own annotation text
            except Exception:  # noqa: BLE001
                return None
    if annotation is Any:
        return Ignore()
    if annotation is int:
        return int_type()
    if annotation is float:
        return float_type()
    if annotation is bool:
        return Boolean()
    if dataclasses.is_dataclass(annotation) and isinstance(annotation, type):
        elements = []
        for field in dataclasses.fields(annotation):
            t = parse_annotation(field.type, glbs)
            if not isinstance(t, Value):
                return None
            elements.append((field.name, t))
        return Structure(annotation, annotation.__name__, tuple(elements))
    origin, args = get_origin(annotation), get_args(annotation)
    if origin is None or len(args) not in (1, 2):
        return None
    element = parse_annotation(args[0], glbs)
    if not isinstance(element, Value):
        return None
    if origin is ptr and len(args) == 1:
        return Pointer(element)
    if origin is grid and len(args) == 2 and type(args[1]) is int:
        return GridType(element, args[1])
    return None


def numpy_dtype(t: Value):
    """numpy dtype of a grid element (xgrid/xgrid/__init__.py:10-18)."""
    import numpy as np
    if isinstance(t, Boolean):
        return np.dtype(np.bool_)
    if isinstance(t, Integer):
        return np.dtype({1: np.int8, 2: np.int16, 4: np.int32, 8: np.int64}[t.width_bytes])
    if isinstance(t, Floating):
        return np.dtype(np.float32 if t.width_bytes == 4 else np.float64)
    if isinstance(t, Structure):
        return np.dtype([(n, numpy_dtype(e)) for n, e in t.elements], align=True)
    raise TypeError(f"no numpy dtype for {t!r}")
