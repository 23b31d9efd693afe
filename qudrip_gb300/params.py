"""The reference's parameter-file reader (find_param.hpp), for drivers that read
`name = value` files the way its programs do.

`param_finder(fname)` reads the file once: every character std::isspace calls
white space is removed from each line, lines starting with '#' or without '='
are skipped, and the first definition of a name wins (find_param.hpp:35-47;
a missing file gives no parameters).  `find_param(name, value, warning=0,
type=...)` returns the converted value, or `value` unchanged when the name is
missing (raising KeyError(name) instead when `warning` is set,
find_param.hpp:59-67).  Conversions follow the C++ ones: floating types parse
the longest leading decimal number as std::stod does, int (and long, which the
reference also reads with std::stoi) the longest leading integer inside the
int32 range, str takes the text, bool is a number's truth value, complex
reads "re", "(re)" or "(re,im)".  `find_param_tvec(name, n, ...)` fills n
values: from the file named after a leading "--" (one value per line, lines
starting with '#' skipped; complex lines hold "re im"), else the one value
repeated (find_param.hpp:83-132).
"""
from __future__ import annotations

import re
from typing import List, Optional

_WS = " \t\n\v\f\r"
_FLOAT = re.compile(r"[+-]?(?:(?:\d+\.?\d*|\.\d+)(?:[eE][+-]?\d+)?|inf(?:inity)?|nan(?:\([0-9A-Za-z_]*\))?)",
                    re.IGNORECASE)
_INT = re.compile(r"[+-]?\d+")


def delete_space(s: str) -> str:
    return "".join(ch for ch in s if ch not in _WS)


def stod(s: str) -> float:
    """std::stod: the longest leading decimal number (after leading white space)."""
    t = s.lstrip(_WS)
    m = _FLOAT.match(t)
    if not m:
        raise ValueError("stod: no conversion")
    return float(m.group(0))


def stoi(s: str) -> int:
    """std::stoi: the longest leading base-10 integer, inside the int32 range."""
    t = s.lstrip(_WS)
    m = _INT.match(t)
    if not m:
        raise ValueError("stoi: no conversion")
    v = int(m.group(0))
    if not -(1 << 31) <= v < (1 << 31):
        raise OverflowError("stoi: out of range")
    return v


def parse_complex(s: str) -> complex:
    """operator>> of std::complex<double>: "re", "(re)" or "(re,im)"."""
    t = s.strip(_WS)
    if t.startswith("("):
        body = t[1:t.index(")")] if ")" in t else t[1:]
        parts = body.split(",")
        if len(parts) == 1:
            return complex(stod(parts[0]), 0.0)
        return complex(stod(parts[0]), stod(parts[1]))
    return complex(stod(t), 0.0)


def convert(text: str, typ):
    if typ is str:
        return text
    if typ is int or typ == "long":
        return stoi(text)
    if typ is bool:
        return bool(stod(text))
    if typ is complex:
        return parse_complex(text)
    return float(stod(text))


class param_finder:
    """find_param.hpp:31-57."""

    def __init__(self, fname: str):
        self.params = {}
        try:
            with open(fname, "r") as f:
                lines = f.read().split("\n")
        except OSError:
            lines = []
        for oline in lines:
            line = delete_space(oline)
            peq = line.find("=")
            if line.startswith("#") or peq < 0:
                continue
            self.params.setdefault(line[:peq], line[peq + 1:])

    def find_param(self, name: str, value=None, warning: int = 0, type=None):
        if name not in self.params:
            if warning:
                raise KeyError(name)
            return value
        typ = type if type is not None else (builtin_type(value) if value is not None else float)
        return convert(self.params[name], typ)

    def find_param_tvec(self, name: str, value: List, warning: int = 0, type=None) -> List:
        """Fills the list `value` in place (its length is the count) and returns it."""
        if name not in self.params:
            if warning:
                raise KeyError(name)
            return value
        typ = type if type is not None else (builtin_type(value[0]) if value else float)
        text = self.params[name]
        if text.startswith("--"):
            with open(text[2:], "r") as f:
                rows = f.read().split("\n")
            it = iter(rows)
            for t in range(len(value)):
                line = ""
                for line in it:
                    if not line.startswith("#"):
                        break
                else:
                    line = ""
                if typ is complex:
                    parts = line.split()
                    value[t] = complex(stod(parts[0]), stod(parts[1]))
                else:
                    value[t] = convert(line, typ)
        else:
            v = convert(text, typ)
            for t in range(len(value)):
                value[t] = v
        return value


def builtin_type(v) -> Optional[type]:
    for t in (bool, int, float, complex, str):
        if isinstance(v, t):
            return t
    return float
