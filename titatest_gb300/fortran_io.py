"""Byte-level emulation of the Fortran output the reference's writers produce.

The reference writes its result files with gfortran, mostly list-directed
(`write(kanal,*) ...`, e.g. src/wdatm.f90:76, src/wout.f90:74-200,
src/wsens.f90:83-93, src/wpot.f90:84) and in a few places with explicit
edit descriptors (src/wout.f90:105 `(7(f10.4,2x))`, :126 `(2(1x,G12.4))`,
:117 `(I7)`).  A Fortran host that diffs its outputs against this library's
needs the same bytes, so the conversions are restated here from the Fortran
standard's edit rules and gfortran's documented list-directed widths:

* every list-directed item is preceded by one blank (for the first item of a
  record that blank is the record's leading blank);
* INTEGER(4): right-justified in 11 columns;
* REAL(4): d = 9 significant digits in a 16-column G-style field: if the
  value rounded to 9 digits lies in [0.1, 1e9) it is written as F12.(9-k)
  followed by 4 blanks (k = digits before the decimal point), zero as F12.8
  plus 4 blanks, otherwise as 1PE16.8E2 (one digit before the point);
* REAL(8): the same with d = 17 in a 25-column field, exponent width 3
  (F20.(17-k) plus 5 blanks, or 1PE25.16E3);
* CHARACTER: the characters as they are.

The decimal conversion is the correctly rounded one of the exact binary
value (round half to even), which is what gfortran's conversion produces.
"""
from __future__ import annotations

import math
from typing import Iterable, Tuple

import numpy as np


def _sig_round(x: float, d: int) -> Tuple[str, int]:
    """Digits (d of them) and decimal exponent e of x rounded to d
    significant digits: |x| ~ 0.digits * 10^(e+1) = d.ddd * 10^e."""
    s = "%.*e" % (d - 1, abs(x))
    mant, exp = s.split("e")
    return mant.replace(".", ""), int(exp)


def _g_list(x: float, d: int, w: int, ew: int) -> str:
    """gfortran list-directed REAL field of width w (without the separator)."""
    if math.isnan(x):
        return "NaN".rjust(w)
    if math.isinf(x):
        return ("-Infinity" if x < 0 else "Infinity").rjust(w)
    neg = math.copysign(1.0, x) < 0
    sign = "-" if neg else ""
    fw = w - (ew + 2)  # width of the F part; ew + 2 blanks stand for the exponent
    if x == 0.0:
        body = sign + "0." + "0" * (d - 1)
        return body.rjust(fw) + " " * (ew + 2)
    digits, e = _sig_round(x, d)
    if -1 <= e < d:  # 0.1 <= |x| < 10^d after rounding: F editing
        k = e + 1  # digits before the decimal point
        if k <= 0:
            body = "0." + digits
        else:
            body = digits[:k] + "." + digits[k:]
        return (sign + body).rjust(fw) + " " * (ew + 2)
    es = "-" if e < 0 else "+"
    body = f"{sign}{digits[0]}.{digits[1:]}E{es}{abs(e):0{ew}d}"
    return body.rjust(w)


def real4(x: float) -> str:
    """One list-directed REAL(4) item (separator blank included)."""
    return " " + _g_list(float(np.float32(x)), 9, 16, 2)


def real8(x: float) -> str:
    """One list-directed REAL(8) item (separator blank included)."""
    return " " + _g_list(float(x), 17, 25, 3)


def int4(i: int) -> str:
    """One list-directed INTEGER(4) item (separator blank included)."""
    return " " + f"{int(i):11d}"


def char(s: str) -> str:
    """One list-directed CHARACTER item (separator blank included)."""
    return " " + s


def record(items: Iterable[str]) -> str:
    """A list-directed record from items made by real4/real8/int4/char."""
    return "".join(items) + "\n"


# ---------------------------------------------------------------------------
# explicit edit descriptors
# ---------------------------------------------------------------------------
def fmt_I(i: int, w: int) -> str:
    s = f"{int(i):d}"
    return "*" * w if len(s) > w else s.rjust(w)


def fmt_F(x: float, w: int, d: int) -> str:
    """Fw.d: rounded to d decimals; a leading zero is dropped when the
    field would otherwise overflow; asterisks when it still does."""
    s = "%.*f" % (d, abs(x))
    if d == 0:
        s += "."  # Fw.0 keeps the decimal point
    neg = math.copysign(1.0, x) < 0 and float(s) != 0.0
    if neg:
        s = "-" + s
    if len(s) > w and (s.startswith("0.") or s.startswith("-0.")):
        s = s.replace("0.", ".", 1)
    return "*" * w if len(s) > w else s.rjust(w)


def fmt_E(x: float, w: int, d: int, e: int = 2) -> str:
    """Ew.dEe with the standard's 0.ddd mantissa (scale factor 0)."""
    if x == 0.0:
        s = "0." + "0" * d + "E+" + "0" * e
        s = ("-" if math.copysign(1.0, x) < 0 else "") + s
        return s.rjust(w)
    digits, ex = _sig_round(x, d)
    ex += 1
    sign = "-" if x < 0 else ""
    s = f"{sign}0.{digits}E{'-' if ex < 0 else '+'}{abs(ex):0{e}d}"
    if len(s) > w and s.startswith(("0.", "-0.")):
        s = s.replace("0.", ".", 1)
    return "*" * w if len(s) > w else s.rjust(w)


def fmt_G(x: float, w: int, d: int, e: int = 2) -> str:
    """Gw.d (no Ee given: the exponent field takes 4 columns): F editing
    F(w-4).(d-k) plus 4 blanks when 0.1 <= |x| < 10^d after rounding to d
    digits, else Ew.d."""
    n = e + 2
    if x == 0.0:
        return fmt_F(x, w - n, d - 1) + " " * n
    digits, ex = _sig_round(x, d)
    if -1 <= ex < d:
        k = ex + 1
        return fmt_F(x, w - n, d - k) + " " * n
    return fmt_E(x, w, d, e)


def tab_record(fields) -> str:
    """A formatted record built with T edit descriptors: fields are
    (column, text) pairs (1-based column); columns never written are
    blanks, and the record ends at the last column written."""
    buf: list = []
    for col, text in fields:
        i = col - 1
        if len(buf) < i + len(text):
            buf.extend(" " * (i + len(text) - len(buf)))
        buf[i:i + len(text)] = list(text)
    return "".join(buf) + "\n"


def fmt_A(s: str, w: int) -> str:
    """Aw output: right-justified when shorter than w, else its first w."""
    return s.rjust(w) if len(s) <= w else s[:w]
