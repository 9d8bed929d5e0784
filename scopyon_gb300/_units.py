"""Unit handling for scopyon configuration leaves.

A scopyon configuration leaf of the form ``{value: v, units: u}`` is read as the
quantity ``v u`` converted to SI base units, and only the magnitude is kept
(reference ``src/scopyon/config.py:101-117``, which delegates the conversion to
pint's ``to_base_units``).  This module restates that conversion for the units
that microscope configurations use: SI prefixes on metre, second, gram, watt,
joule, newton, hertz, molar and mole; radian and degree; ``dimensionless``; and
products, quotients and integer powers of those (``kg / s ** 3``, ``W/m^2``).
"""

import math
import re

__all__ = ["Quantity", "DimensionalityError", "parse_units", "to_base_magnitude"]

# dimension vector order: metre, kilogram, second, ampere, kelvin, mole, candela, radian
_DIMS = 8


def _dim(**kw):
    order = ("m", "kg", "s", "A", "K", "mol", "cd", "rad")
    return tuple(kw.get(k, 0) for k in order)


_NONE = _dim()

# name -> (factor to SI base, dimension vector)
_BASE = {
    "m": (1.0, _dim(m=1)), "meter": (1.0, _dim(m=1)), "metre": (1.0, _dim(m=1)),
    "s": (1.0, _dim(s=1)), "sec": (1.0, _dim(s=1)), "second": (1.0, _dim(s=1)),
    "min": (60.0, _dim(s=1)), "minute": (60.0, _dim(s=1)), "h": (3600.0, _dim(s=1)),
    "hour": (3600.0, _dim(s=1)),
    "g": (1e-3, _dim(kg=1)), "gram": (1e-3, _dim(kg=1)),
    "A": (1.0, _dim(A=1)), "ampere": (1.0, _dim(A=1)),
    "K": (1.0, _dim(K=1)), "kelvin": (1.0, _dim(K=1)),
    "mol": (1.0, _dim(mol=1)), "mole": (1.0, _dim(mol=1)),
    "M": (1e3, _dim(mol=1, m=-3)), "molar": (1e3, _dim(mol=1, m=-3)),
    "cd": (1.0, _dim(cd=1)), "candela": (1.0, _dim(cd=1)),
    "rad": (1.0, _dim(rad=1)), "radian": (1.0, _dim(rad=1)),
    "deg": (math.pi / 180.0, _dim(rad=1)), "degree": (math.pi / 180.0, _dim(rad=1)),
    "W": (1.0, _dim(kg=1, m=2, s=-3)), "watt": (1.0, _dim(kg=1, m=2, s=-3)),
    "J": (1.0, _dim(kg=1, m=2, s=-2)), "joule": (1.0, _dim(kg=1, m=2, s=-2)),
    "N": (1.0, _dim(kg=1, m=1, s=-2)), "newton": (1.0, _dim(kg=1, m=1, s=-2)),
    "Hz": (1.0, _dim(s=-1)), "hertz": (1.0, _dim(s=-1)),
    "L": (1e-3, _dim(m=3)), "l": (1e-3, _dim(m=3)), "liter": (1e-3, _dim(m=3)),
    "litre": (1e-3, _dim(m=3)),
    "dimensionless": (1.0, _NONE), "percent": (1e-2, _NONE), "count": (1.0, _NONE),
}

_PREFIX = {
    "Y": 1e24, "Z": 1e21, "E": 1e18, "P": 1e15, "T": 1e12, "G": 1e9, "M": 1e6, "k": 1e3,
    "h": 1e2, "da": 1e1, "d": 1e-1, "c": 1e-2, "m": 1e-3, "u": 1e-6, "µ": 1e-6,
    "μ": 1e-6, "n": 1e-9, "p": 1e-12, "f": 1e-15, "a": 1e-18,
}
_LONG_PREFIX = {
    "yotta": 1e24, "zetta": 1e21, "exa": 1e18, "peta": 1e15, "tera": 1e12, "giga": 1e9,
    "mega": 1e6, "kilo": 1e3, "hecto": 1e2, "deca": 1e1, "deci": 1e-1, "centi": 1e-2,
    "milli": 1e-3, "micro": 1e-6, "nano": 1e-9, "pico": 1e-12, "femto": 1e-15, "atto": 1e-18,
}


class DimensionalityError(ValueError):
    """Raised when a quantity is assigned where another dimension is expected."""

    def __init__(self, units1, units2, dim1=None, dim2=None):
        super().__init__("Cannot convert from '%s' to '%s'" % (units1, units2))
        self.units1, self.units2, self.dim1, self.dim2 = units1, units2, dim1, dim2


def _lookup(name):
    if name in _BASE:
        return _BASE[name]
    plural = name[:-1] if name.endswith("s") and name[:-1] in _BASE and len(name) > 2 else None
    if plural:
        return _BASE[plural]
    for pre, fac in _LONG_PREFIX.items():
        if name.startswith(pre) and name[len(pre):]:
            f, d = _lookup(name[len(pre):])
            return fac * f, d
    for pre in sorted(_PREFIX, key=len, reverse=True):
        rest = name[len(pre):]
        if name.startswith(pre) and rest in _BASE:
            f, d = _BASE[rest]
            return _PREFIX[pre] * f, d
    raise ValueError("unknown unit %r" % name)


_TOKEN = re.compile(r"\s*(\*\*|\^|\*|/|\(|\)|-|[0-9]+(?:\.[0-9]*)?(?:[eE][-+]?[0-9]+)?|[A-Za-zµμ_]+)")


def parse_units(text):
    """Return ``(factor, dims)`` for a unit expression such as ``'kg / s ** 3'``."""
    if text is None:
        return 1.0, _NONE
    text = str(text).strip()
    if not text:
        return 1.0, _NONE
    tokens, pos = [], 0
    while pos < len(text):
        m = _TOKEN.match(text, pos)
        if not m or m.end() == pos:
            raise ValueError("cannot parse units %r" % text)
        tokens.append(m.group(1))
        pos = m.end()
        while pos < len(text) and text[pos].isspace():
            pos += 1
    state = {"i": 0}

    def peek():
        return tokens[state["i"]] if state["i"] < len(tokens) else None

    def take():
        tok = tokens[state["i"]]
        state["i"] += 1
        return tok

    def atom():
        tok = take()
        if tok == "(":
            val = expr()
            if take() != ")":
                raise ValueError("unbalanced parentheses in %r" % text)
        elif re.match(r"[0-9]", tok):
            val = (float(tok), _NONE)
        else:
            val = _lookup(tok)
        if peek() in ("**", "^"):
            take()
            sign = 1
            if peek() == "-":
                take()
                sign = -1
            power = sign * float(take())
            if power != int(power):
                raise ValueError("non-integer unit power in %r" % text)
            power = int(power)
            val = (val[0] ** power, tuple(d * power for d in val[1]))
        return val

    def expr():
        fac, dims = atom()
        while peek() in ("*", "/") or (peek() is not None and peek() not in (")",)):
            op = take() if peek() in ("*", "/") else "*"
            f2, d2 = atom()
            if op == "*":
                fac, dims = fac * f2, tuple(a + b for a, b in zip(dims, d2))
            else:
                fac, dims = fac / f2, tuple(a - b for a, b in zip(dims, d2))
        return fac, dims

    out = expr()
    if state["i"] != len(tokens):
        raise ValueError("cannot parse units %r" % text)
    return out


def to_base_magnitude(value, units):
    """Convert ``value`` (a number or a nested list of numbers) in ``units`` to SI."""
    factor, _ = parse_units(units)
    if value is None:
        return None
    if isinstance(value, (list, tuple)):
        return [to_base_magnitude(v, units) for v in value]
    return value * factor if factor != 1.0 else value


class Quantity:
    """A value with units, accepted by ``Configuration.__setattr__``.

    Mirrors the role of ``scopyon.constants.Quantity`` (a pint quantity): the
    assignment keeps the value and unit string and checks that its dimension
    matches the leaf it replaces.
    """

    def __init__(self, magnitude, units="dimensionless"):
        self.magnitude = magnitude
        self.units = units
        parse_units(units)

    @property
    def dimensionality(self):
        return parse_units(self.units)[1]

    def check(self, other_units):
        return parse_units(other_units)[1] == self.dimensionality

    def to_base_units(self):
        return to_base_magnitude(self.magnitude, self.units)

    def __repr__(self):
        return "Quantity(%r, %r)" % (self.magnitude, self.units)
