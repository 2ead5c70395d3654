"""Pragma stubs recognised by the parser (xgrid/lang/__init__.py:1-17).

``with xgrid.boundary(k):`` selects the mask value of the sweeps written inside
it; ``with xgrid.c():`` turns string statements into inline source.  At run time
both are no-op context managers.
"""


class StubContext:
    def __enter__(self):
        return None

    def __exit__(self, *exc):
        return False


def c() -> StubContext:
    return StubContext()


def boundary(type: int) -> StubContext:  # noqa: A002 - reference keyword name
    return StubContext()
