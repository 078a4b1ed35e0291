"""Tier-1 oracle: executes the reference's generated Gaussian-integral code.

TEST INFRASTRUCTURE ONLY.  Nothing in the product imports this module; it is
used by ``tests/golden/make_primitive_goldens.py`` to turn the reference's own
straight-line Fortran (``src/olcao/gaussIntegrals.f90``) into golden vectors,
and by CPU tests that re-check those vectors when the reference tree is
present.

The reference file is machine generated: every integral subroutine is a short
header of prefactor statements followed by ``if (l1l2switch .eq. N)`` blocks
of scalar assignments to ``pc(..)``/``pc_ol(..)``/``sh(..)``.  This module
parses exactly that subset of Fortran 90 and interprets it with Python
binary64 floats, so the values it produces carry the reference's own
arithmetic and operation order:

* ``overlap2CIntg``   gaussIntegrals.f90:26-4420
* ``kinetic2CIntg``   gaussIntegrals.f90:4422-11622
* ``electron3CIntg``  gaussIntegrals.f90:11624-16023
* ``boys``            gaussIntegrals.f90:16080-16221
* ``nuclear3CIntg``   gaussIntegrals.f90:16223-23039
* ``momentum2CIntg``  gaussIntegrals.f90:23041-39068 (sh(16,16,3))

Fortran typing rules that change results are honoured: a real literal with a
``d`` exponent is double precision, a real literal without one is a
default-kind (single precision) constant that is rounded to binary32 before
use (this matters for the Boys-series constants at gaussIntegrals.f90:
16117-16190, which the gfortran build of the reference stores as REAL(4)).
"""

from __future__ import annotations

import math
import os
import re
from typing import Dict, List, Tuple

import numpy as np

PI = 3.141592653589793  # src/constants.f90:36

_SUBROUTINES = ("overlap2CIntg", "kinetic2CIntg", "electron3CIntg",
                "nuclear3CIntg", "massvel2CIntg", "momentum2CIntg", "boys")
# fineStructure of src/constants.f90:47 (in units of 1e-3), the only
# module constant besides pi that the generated integrals read
FINE_STRUCTURE = 7.2973525693
_FUNCS = {"exp": "_exp", "sqrt": "_sqrt", "sum": "_sum", "erf": "_erf",
          "abs": "abs"}
_VECTORS = {"p", "pa", "pb", "g", "ga", "gb", "gc", "pc_3c", "d", "d1", "d2",
            "d3", "a", "b", "c"}


def _f32(x: float) -> float:
    return float(np.float32(x))


def _exp(x):
    return np.exp(x) if isinstance(x, np.ndarray) else math.exp(x)


def _sqrt(x):
    return np.sqrt(x) if isinstance(x, np.ndarray) else math.sqrt(x)


def _sum(x):
    return float(np.sum(x))


def _erf(x):
    return math.erf(x)


_TOKEN = re.compile(r"""
    (?P<num>(\d+\.\d*|\.\d+|\d+)([dDeE][-+]?\d+)?)
  | (?P<name>[A-Za-z_][A-Za-z_0-9]*)
  | (?P<op>\*\*|[-+*/(),=:])
  | (?P<ws>\s+)
""", re.VERBOSE)


def _literal(tok: str) -> str:
    """Return Python source for a Fortran numeric literal."""
    low = tok.lower()
    if "d" in low:
        return repr(float(low.replace("d", "e")))
    if "." in low or "e" in low:
        return repr(_f32(float(low)))   # default REAL kind: binary32
    return str(int(low))


def _translate(expr: str) -> str:
    """Translate one Fortran expression into Python source."""
    out: List[str] = []
    pos = 0
    toks: List[Tuple[str, str]] = []
    while pos < len(expr):
        m = _TOKEN.match(expr, pos)
        if not m:
            raise ValueError(f"cannot tokenize {expr[pos:]!r}")
        pos = m.end()
        kind = m.lastgroup
        if kind == "ws":
            continue
        toks.append((kind, m.group(kind)))
    i = 0
    while i < len(toks):
        kind, val = toks[i]
        nxt = toks[i + 1][1] if i + 1 < len(toks) else None
        if kind == "num":
            out.append(_literal(val))
        elif kind == "name":
            val = val.lower()
            if nxt == "(" and val in _FUNCS:
                out.append(_FUNCS[val.lower()])
            elif nxt == "(":
                # array element: name(i,j,...) -> name[(i,j,...)]
                depth = 0
                j = i + 1
                inner: List[Tuple[str, str]] = []
                while True:
                    t = toks[j]
                    if t[1] == "(":
                        depth += 1
                        if depth > 1:
                            inner.append(t)
                    elif t[1] == ")":
                        depth -= 1
                        if depth == 0:
                            break
                        inner.append(t)
                    else:
                        inner.append(t)
                    j += 1
                src = " ".join(_literal(v) if k == "num" else
                               (v.lower() if k == "name" else v)
                               for k, v in inner)
                if src.strip() == ":":
                    out.append(val)            # whole-array section name(:)
                elif val in _VECTORS:
                    out.append(f"{val}[({src})-1]")
                else:
                    out.append(f"{val}[({src},)]")
                i = j
            else:
                out.append(val)
        else:
            out.append(val)
        i += 1
    return " ".join(out)


def _logical_lines(lines: List[str]) -> List[str]:
    """Join '&' continuations and strip comments."""
    res: List[str] = []
    buf = ""
    for raw in lines:
        line = raw.split("!", 1)[0].rstrip()
        if not line.strip():
            continue
        s = line.strip()
        if buf:
            if s.startswith("&"):
                s = s[1:]
            buf += s
        else:
            buf = s
        if buf.endswith("&"):
            buf = buf[:-1]
            continue
        res.append(buf)
        buf = ""
    return res


_SKIP = re.compile(r"^(use|implicit|real|integer|end\s+subroutine|subroutine|"
                   r"contains|module|public)\b", re.I)


def _compile(stmts: List[str]) -> str:
    """Compile a list of Fortran statements into Python function body source."""
    py: List[str] = []
    ind = 1
    for s in stmts:
        low = s.lower().strip()
        if _SKIP.match(low):
            continue
        m = re.match(r"^(else\s*if)\s*\((.*)\)\s*then$", low)
        if m:
            ind -= 1
            cond = s[s.index("(") + 1:s.rindex(")")]
            py.append("    " * ind + f"elif {_translate_cond(cond)}:")
            ind += 1
            continue
        if re.match(r"^if\s*\(.*\)\s*then$", low):
            cond = s[s.index("(") + 1:s.rindex(")")]
            py.append("    " * ind + f"if {_translate_cond(cond)}:")
            ind += 1
            continue
        if low == "else":
            py.append("    " * (ind - 1) + "else:")
            continue
        if low in ("end if", "endif"):
            py.append("    " * ind + "pass")
            ind -= 1
            continue
        m = re.match(r"^do\s+(\w+)\s*=\s*(.+),\s*(.+)$", low)
        if m:
            v, a, b = m.groups()
            py.append("    " * ind +
                      f"for {v} in range({_translate(a)}, {_translate(b)} + 1):")
            ind += 1
            continue
        if low in ("end do", "enddo"):
            py.append("    " * ind + "pass")
            ind -= 1
            continue
        m = re.match(r"^call\s+boys\s*\(\s*(\w+)\s*,\s*(\w+)\s*\)$", low)
        if m:
            py.append("    " * ind + f"{m.group(2)} = _boys({m.group(1)})")
            continue
        if "=" in s:
            lhs, rhs = s.split("=", 1)
            lhs_t = _translate(lhs.strip())
            py.append("    " * ind + f"{lhs_t} = {_translate(rhs.strip())}")
            continue
        raise ValueError(f"unsupported statement: {s}")
    return "\n".join(py)


def _translate_cond(cond: str) -> str:
    c = cond.replace(".eq.", " == ").replace(".le.", " <= ")
    # split on comparison operators so each side is translated separately
    parts = re.split(r"(==|<=|>=|<|>)", c)
    return " ".join(p if p in ("==", "<=", ">=", "<", ">") else _translate(p)
                    for p in parts)


class FortranIntegrals:
    """Interprets the reference's generated integral subroutines."""

    def __init__(self, path: str):
        with open(path) as fh:
            src = fh.readlines()
        self._subs: Dict[str, object] = {}
        for name in _SUBROUTINES:
            start = end = None
            for i, line in enumerate(src):
                low = line.strip().lower()
                if start is None and re.match(rf"subroutine\s+{name.lower()}\s*\(", low):
                    start = i
                elif start is not None and re.match(rf"end\s+subroutine\s+{name.lower()}", low):
                    end = i
                    break
            if start is None or end is None:
                raise ValueError(f"{name} not found in {path}")
            self._subs[name] = (start + 1, end + 1)
            stmts = _logical_lines(src[start:end + 1])
            body = _compile(stmts)
            args = {"overlap2CIntg": "a1, a2, a, b, l1l2switch",
                    "kinetic2CIntg": "a1, a2, a, b, l1l2switch",
                    "electron3CIntg": "a1, a2, a3, a, b, c, l1l2switch",
                    "nuclear3CIntg": "a1, a2, a3, a, b, c, l1l2switch",
                    "massvel2CIntg": "a1, a2, a, b, l1l2switch",
                    "momentum2CIntg": "a1, a2, a, b, l1l2switch",
                    "boys": "t"}[name]
            if name == "boys":
                pre = "    s = {}\n    f = {}\n"
                post = "\n    return [f[(m,)] for m in range(1, 8)]"
            else:
                pre = ("    pc = {}\n    pc_ol = {}\n    pc_ke = {}\n    sh = {}\n"
                       "    prefactorn = {}\n    prefactormm = {}\n    f = {}\n")
                post = "\n    return sh"
            code = f"def _{name}({args}):\n{pre}{body}{post}\n"
            ns = {"_exp": _exp, "_sqrt": _sqrt, "_sum": _sum, "_erf": _erf,
                  "pi": PI, "finestructure": FINE_STRUCTURE, "np": np, "math": math}
            exec(compile(code, f"<{name}>", "exec"), ns)
            self.__dict__["_fn_" + name] = ns["_" + name]
            if name == "boys":
                self._boys_fn = ns["_boys"]
        # nuclear3CIntg calls boys: bind it into that function's globals
        for name in ("nuclear3CIntg",):
            fn = self.__dict__["_fn_" + name]
            fn.__globals__["_boys"] = self._boys_list

    def _boys_list(self, T):
        vals = self._boys_fn(float(T))
        return {(m + 1,): v for m, v in enumerate(vals)}

    def line_span(self, name: str) -> Tuple[int, int]:
        return self._subs[name]

    def boys(self, T: float) -> List[float]:
        return self._boys_fn(float(T))

    def _run(self, name, *args) -> np.ndarray:
        sh = self.__dict__["_fn_" + name](*args)
        out = np.full((16, 16), np.nan)
        for (i, j), v in sh.items():
            out[i - 1, j - 1] = v
        return out

    def overlap(self, a1, a2, A, B, switch):
        return self._run("overlap2CIntg", float(a1), float(a2),
                         np.asarray(A, float), np.asarray(B, float), int(switch))

    def kinetic(self, a1, a2, A, B, switch):
        return self._run("kinetic2CIntg", float(a1), float(a2),
                         np.asarray(A, float), np.asarray(B, float), int(switch))

    def massvel(self, a1, a2, A, B, switch):
        return self._run("massvel2CIntg", float(a1), float(a2),
                         np.asarray(A, float), np.asarray(B, float), int(switch))

    def momentum(self, a1, a2, A, B, switch):
        """momentum2CIntg: sh(16,16,3), the x, y, z components."""
        sh = self.__dict__["_fn_momentum2CIntg"](float(a1), float(a2), np.asarray(A, float),
                                                   np.asarray(B, float), int(switch))
        out = np.full((16, 16, 3), np.nan)
        for (i, j, c), v in sh.items():
            out[i - 1, j - 1, c - 1] = v
        return out

    def electron3c(self, a1, a2, a3, A, B, C, switch):
        return self._run("electron3CIntg", float(a1), float(a2), float(a3),
                         np.asarray(A, float), np.asarray(B, float),
                         np.asarray(C, float), int(switch))

    def nuclear3c(self, a1, a2, a3, A, B, C, switch):
        return self._run("nuclear3CIntg", float(a1), float(a2), float(a3),
                         np.asarray(A, float), np.asarray(B, float),
                         np.asarray(C, float), int(switch))


def l1l2switch(lmalpha1: int, lmalpha2: int) -> int:
    """Opcode of integrals.F90:387-390: 2**p(lmAlpha1) + 16*2**p(lmAlpha2)."""
    p = {1: 0, 4: 1, 9: 2, 16: 3}
    return (1 << p[lmalpha1]) + (16 << p[lmalpha2])


def default_path() -> str:
    return os.environ.get(
        "OLCAO_REFERENCE_GAUSS",
        "/root/reference/src/olcao/gaussIntegrals.f90")
