"""``@xgrid.kernel`` / ``@xgrid.function`` / ``@xgrid.external`` operators.

Call protocol of xgrid/lang/operator.py:13-64: a kernel parses and compiles on
its first call, then on every call ticks each ``Grid`` argument to the kernel's
time depth (in argument order) and invokes the native entry point.  Here the
native entry point is the generated CUDA module, called through the runtime's
graph cache (``xg_call``) on the backend stream; the call is asynchronous except
for kernels that return a value.
"""
from __future__ import annotations

from typing import Any, Callable

from . import ir
from .log import Logger
from .types import BaseType

CustomTypecheck = Callable[[list], BaseType]


class Operator:
    def __init__(self, func, mode: str, name: str | None = None, includes: list | None = None,
                 self_type: BaseType | None = None, typecheck_override: CustomTypecheck | None = None,
                 tick: bool = True, macro: list | None = None) -> None:
        self.func = func
        self.mode = mode
        self.logger = Logger(self)
        self.name = func.__name__ if name is None else name
        self.includes = [] if includes is None else list(includes)
        self.macro = [] if macro is None else list(macro)
        self.native = None
        self.self_type = self_type
        self.typecheck_override = typecheck_override
        self.tick = tick

    def __call__(self, *args: Any) -> Any:
        if self.mode == "kernel":
            if self.native is None:
                from .native import NativeKernel
                self.native = NativeKernel(self)
            return self.native(*args)
        if self.mode == "function":
            return self.func(*args)
        self.logger.dead(f"Invalid call to non-kernel or non-function ({self.mode}) operator '{self.name}'")

    def batch(self, problems, steps: int = 1, temporal=None) -> None:
        """Run ``steps`` calls of this kernel on each of ``problems`` (argument
        tuples of independent problems) with one persistent launch per step, or
        per ``depth`` steps when the kernel can be temporally blocked
        (``temporal``: ``(depth, ty, tx)``, 1 for none; default: the kernel's
        setting, else the tuned or built-in one)."""
        if self.mode != "kernel":
            self.logger.dead(f"Only kernels can be batched, '{self.name}' is a {self.mode}")
        if self.native is None:
            from .native import NativeKernel
            self.native = NativeKernel(self)
        return self.native.batch(problems, steps, temporal)

    @property
    def ir(self) -> ir.Definition:
        cached = getattr(self, "_ir", None)
        if cached is None:
            from .parser import Parser
            parser = Parser(self.func, self.name, self.mode, self.self_type)
            self._ir = cached = parser.result
            self.includes.extend(i for i in parser.includes if i not in self.includes)
        return cached

    @property
    def src(self) -> str:
        """Generated CUDA source of this kernel."""
        from .codegen import CudaGenerator
        from .config import get_config
        return CudaGenerator(self, get_config()).generate().source

    @property
    def signature(self) -> ir.Signature:
        return self.ir.signature


def kernel(*, name: str | None = None, includes: list | None = None, tick: bool = True,
           macro: list | None = None, noalloc: bool = False):
    """``noalloc=True`` also compiles ``xg_kernel_<name>_noalloc``, a variant of
    the module's entry point whose scratch buffers come from a fixed device pool
    instead of the caller (see ``include/xgrid_gb300.h``)."""
    def aux(func):
        op = Operator(func, "kernel", name, includes, tick=tick, macro=macro)
        op.noalloc = noalloc
        return op
    return aux


def function(*, method: bool = False, name: str | None = None, includes: list | None = None,
             macro: list | None = None):
    if method:
        def aux_method(func):
            setattr(func, "__xgrid_method", (name, includes))
            return func
        return aux_method

    def aux(func):
        return Operator(func, "function", name, includes, macro=macro)
    return aux


def external(*, name: str | None = None, includes: list | None = None, typecheck_override: CustomTypecheck):
    def aux(func):
        return Operator(func, "external", name, includes, typecheck_override=typecheck_override)
    return aux
