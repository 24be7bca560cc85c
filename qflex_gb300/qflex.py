"""Drop-in for the reference's Python module ``qflex`` (pybind entry
``qflex.simulate``, src/pybind_main.h:19-23, src/pybind_main.cpp:75-138).

``simulate(options)`` takes the same dict and returns the same
``list[tuple[str, complex]]``; the contraction runs on the GB300 engine
through the C ABI. As in the reference, input errors are printed to stderr
and an empty list is returned; any other failure is raised.
"""
from __future__ import annotations

import re
import sys
import threading
from typing import Iterable, List, Optional, Tuple

from ._lib import ERR_INPUT, FP32, Context, QflexGb300Error

_DEFAULT_LIMIT = 1 << 30
_state = threading.local()
_memory_limit = [_DEFAULT_LIMIT]  # global::memory_limit (src/global.h:12)


class _InputError(Exception):
    pass


def default_context() -> Context:
    """The module's engine context on CUDA device 0 (created on first use)."""
    ctx = getattr(_state, "ctx", None)
    if ctx is None:
        ctx = Context(0, FP32)
        _state.ctx = ctx
    return ctx


def set_default_context(ctx: Optional[Context]) -> None:
    _state.ctx = ctx


def from_readable_memory_string(s: str) -> int:
    """utils::from_readable_memory_string (src/utils.cpp:19-57)."""
    s = re.sub(r"[^)(\s\ta-zA-Z0-9_.,-]", "", s).replace("\t", " ").replace(" ", "").upper()
    m = re.match(r"^(\d+)(.*)$", s)
    if not m:
        raise _InputError(f"Memory string '{s}' must start with a number.")
    value, suffix = int(m.group(1)), m.group(2)
    scale = {"GB": 1 << 30, "MB": 1 << 20, "KB": 1 << 10, "B": 1, "": 1}
    if suffix not in scale:
        raise _InputError(f"Suffix {suffix} not recognized.")
    return value * scale[suffix]


def _stream_text(data, caller: str) -> str:
    # GetStream (src/pybind_main.cpp:8-17): one line per element.
    out = []
    for line in data:
        if not isinstance(line, str):
            raise _InputError(f"{caller} must be a list of strings.")
        out.append(line + "\n")
    return "".join(out)


def _load_text(options: dict, argument: str) -> str:
    # LoadData (src/pybind_main.cpp:26-42).
    if argument in options:
        data = options[argument]
        if not isinstance(data, Iterable):
            raise _InputError(f"'{argument}' must be a list of strings.")
        return _stream_text(data, argument)
    key = argument + "_filename"
    if key in options:
        name = options[key]
        if not isinstance(name, str):
            raise _InputError(f"'{argument}_filename' must be a string.")
        try:
            with open(name) as f:
                return f.read()
        except OSError:
            what = {"circuit": "Cannot open circuit file ", "grid": "Cannot open grid file: ",
                    "ordering": "Cannot open ordering file: "}[argument]
            raise _InputError(f"{what}{name}{'.' if argument != 'ordering' else ''}")
    return ""


def _load_states(options: dict, argument: str) -> List[str]:
    # LoadStates (src/pybind_main.cpp:49-73).
    if argument + "_states" in options:
        v = options[argument + "_states"]
        if isinstance(v, str):
            return [v]
        if isinstance(v, Iterable):
            out = []
            for x in v:
                if not isinstance(x, str):
                    raise _InputError("states must be strings.")
                out.append(x)
            return out
        raise _InputError(f"{argument}_states must be a list of strings.")
    if argument + "_state" in options:
        v = options[argument + "_state"]
        if not isinstance(v, str):
            raise _InputError("states must be strings.")
        return [v]
    return [""]


def simulate(options: dict, context: Optional[Context] = None) -> List[Tuple[str, complex]]:
    """qflex.simulate: evaluate the amplitudes the ordering asks for."""
    try:
        if "memory_limit" in options:
            ml = options["memory_limit"]
            if isinstance(ml, bool) or not isinstance(ml, (int, str)):
                pass  # the reference builds an error message but does not throw
            elif isinstance(ml, int):
                if ml <= 0:
                    raise _InputError("'memory_limit' must be positive.")
                _memory_limit[0] = ml
            else:
                _memory_limit[0] = from_readable_memory_string(ml)
        else:
            _memory_limit[0] = _DEFAULT_LIMIT
        grid = _load_text(options, "grid")
        circuit = _load_text(options, "circuit")
        ordering = _load_text(options, "ordering")
        initial = _load_states(options, "initial")
        final = _load_states(options, "final")
        if len(initial) != 1 or len(final) != 1:
            raise _InputError("Not yet supported")
        ctx = context or default_context()
        return ctx.evaluate(circuit, ordering, grid, initial[0], final[0], float(_memory_limit[0]))
    except _InputError as e:
        print(f"ERROR (qflex_gb300: simulate) --> {e}", file=sys.stderr)
    except QflexGb300Error as e:
        if e.code != ERR_INPUT:
            raise
        print(str(e), file=sys.stderr)
    return []
