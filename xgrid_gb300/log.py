"""Leveled logger whose ``dead`` raises ``Exception``.

Behaviour follows the reference's error convention (xgrid/util/logging.py:22-60):
every front-end, compile or launch error is logged at level ``dead`` and then
raised as a plain ``Exception`` whose ``args`` are the message lines.  Sinks are
class-level lists of text streams that tests may swap for ``io.StringIO``.
"""
from __future__ import annotations

import enum
import sys
from typing import NoReturn, TextIO


class LogLevel(enum.IntEnum):
    info = 0
    done = 1
    warn = 2
    fail = 3
    dead = 4


_COLOURS = {LogLevel.info: 34, LogLevel.done: 32, LogLevel.warn: 33,
            LogLevel.fail: 31, LogLevel.dead: 35}


class Logger:
    """Per-object logger.  ``stdouts`` receive info/done, ``stderrs`` the rest."""

    stdouts: list[TextIO] = [sys.stdout]
    stderrs: list[TextIO] = [sys.stderr]
    level: LogLevel = LogLevel.warn

    def __init__(self, owner: object | str) -> None:
        if isinstance(owner, str):
            self.name = owner
        else:
            self.name = f"{type(owner).__module__}.{type(owner).__qualname__}@{id(owner)}"

    def log(self, level: LogLevel, *msg: str) -> None:
        if level < Logger.level:
            return
        targets = Logger.stdouts if level <= LogLevel.done else Logger.stderrs
        for target in targets:
            tty = getattr(target, "isatty", lambda: False)()
            tag = f"\033[1;{_COLOURS[level]}m{level.name}\033[0m" if tty else level.name
            for i, line in enumerate(msg):
                target.write((f"[ {tag} | {self.name} ] {line}" if i == 0 else line) + "\n")

    def info(self, *msg: str) -> None:
        self.log(LogLevel.info, *msg)

    def done(self, *msg: str) -> None:
        self.log(LogLevel.done, *msg)

    def warn(self, *msg: str) -> None:
        self.log(LogLevel.warn, *msg)

    def fail(self, *msg: str) -> None:
        self.log(LogLevel.fail, *msg)

    def dead(self, *msg: str) -> NoReturn:
        self.log(LogLevel.dead, *msg)
        raise Exception(msg)
