"""The reference's result-file formats for what this engine computes.

``rXXForceNonDim.csv`` (src/libPostprocess.f90:33-36 header, :814-833 rows):
a header ``(A5, 9(A15))`` and per written step the zero-padded iteration
``(I0.5)`` followed by nine ``E15.7`` values -- CL/CT, CD/CQ, CLu, CDi, CD0,
CDu, CFx, CFy, CFz -- exactly the ten columns ``vlm_case_step`` returns per
step, so the reference's post-processing tools read these files unchanged.
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Iterable, Sequence

FORCE_NONDIM_COLUMNS = ("iter", "CL/CT", "CD/CQ", "CLu", "CDi", "CD0", "CDu", "CFx", "CFy", "CFz")


def fortran_e(x: float, width: int = 15, digits: int = 7) -> str:
    """Fortran ``Ew.d`` output: ``0.ddddddd``E+ee`` (mantissa in [0.1, 1)),
    right-justified in ``width`` characters."""
    if x == 0.0 or not math.isfinite(x):
        body = ("0." + "0" * digits + "E+00") if x == 0.0 else ("NaN" if x != x else ("Infinity" if x > 0 else "-Infinity"))
        return body.rjust(width)
    sign = "-" if x < 0 else ""
    a = abs(x)
    e = math.floor(math.log10(a)) + 1
    m = round(a / 10.0 ** e, digits)
    if m >= 1.0:  # rounding carried into the next decade
        m /= 10.0
        e += 1
    if m < 0.1:
        m *= 10.0
        e -= 1
    mant = f"{m:.{digits}f}"
    if mant.startswith("1"):  # 0.99999995 rounds up
        mant = f"{0.1:.{digits}f}"
        e += 1
    exp = f"E{'+' if e >= 0 else '-'}{abs(e):02d}"
    return (sign + mant + exp).rjust(width)


def force_nondim_header() -> str:
    return FORCE_NONDIM_COLUMNS[0].rjust(5) + "".join(c.rjust(15) for c in FORCE_NONDIM_COLUMNS[1:])


def force_nondim_line(row: Sequence[float]) -> str:
    """One data line from a 10-column CT row (iteration first)."""
    return f"{int(round(row[0])):05d}" + "".join(fortran_e(float(v)) for v in row[1:10])


def write_force_nondim(path, rows: Iterable[Sequence[float]], header: bool = True) -> Path:
    """Writes (or appends to, header=False) an rXXForceNonDim.csv file."""
    p = Path(path)
    with open(p, "w" if header else "a") as f:
        if header:
            f.write(force_nondim_header() + "\n")
        for r in rows:
            f.write(force_nondim_line(r) + "\n")
    return p
