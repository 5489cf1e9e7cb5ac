"""The reference's result-file formats for what this engine computes.

``rXXForceNonDim.csv`` (src/libPostprocess.f90:33-36 header, :814-833 rows):
a header ``(A5, 9(A15))`` and per written step the zero-padded iteration
``(I0.5)`` followed by nine ``E15.7`` values -- CL/CT, CD/CQ, CLu, CDi, CD0,
CDu, CFx, CFy, CFz -- exactly the ten columns ``vlm_case_step`` returns per
step, so the reference's post-processing tools read these files unchanged.

``rXXForceDim.csv`` (header ``(A5, 11(A15))``, rows ``(A, 11(E15.7))``,
src/libPostprocess.f90:27-31,840-846), ``rXXbYYForceDistNNNNN.csv`` (one file
per blade and written iteration: a ``16(A15)`` header and ns ``16(E15.7)``
rows, :848-881), ``rXXParams.json`` (params2file, :52-141; the text comes
from the library) and the ``rXXbladedynamics.csv`` header (:39-42) complete
the Results/ directory of a run: :class:`ResultsWriter` writes them at the
iterations the reference does (src/main.f90:39,238-241,341,624-719).
"""
from __future__ import annotations

import math
from pathlib import Path
from typing import Iterable, Sequence

import numpy as np

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


FORCE_DIM_COLUMNS = ("iter", "LiftMag", "DragMag", "Lx", "Ly", "Lz", "Dx", "Dy", "Dz", "FInertx", "FInerty", "FInertz")
FORCE_DIST_COLUMNS = ("secSpan", "secCL", "secCD", "secCLu", "secLift", "secDrag", "secLiftInPl", "secLiftOutPl",
                      "secArea", "secVel", "secChord", "secTheta", "secAlpha", "secPhi", "secViz", "secVix")
DYNAMICS_COLUMNS = ("iter", "pitch", "flap", "dflap", "w", "omega")


def _header(cols: Sequence[str], first: int = 5) -> str:
    return cols[0].rjust(first) + "".join(c.rjust(15) for c in cols[1:])


def force_dim_header() -> str:
    return _header(FORCE_DIM_COLUMNS)


def force_dim_line(iteration: int, values: Sequence[float]) -> str:
    """One rXXForceDim.csv line: |L|, |D|, L, D, forceInertial (11 values)."""
    return f"{int(iteration):05d}" + "".join(fortran_e(float(v)) for v in values[:11])


def force_dist_text(dist) -> str:
    """A whole rXXbYYForceDistNNNNN.csv file from an (ns, 16) array."""
    lines = ["".join(c.rjust(15) for c in FORCE_DIST_COLUMNS)]
    lines += ["".join(fortran_e(float(v)) for v in row) for row in dist]
    return "\n".join(lines) + "\n"


def dynamics_header() -> str:
    return _header(DYNAMICS_COLUMNS)


class ResultsWriter:
    """The Results/ files of one rotor case, written as the reference's main
    program writes them.

    ``start()`` (after ``Case.start()``): rXXParams.json, the headers of the
    force and dynamics files, and the iteration-0 force rows and sectional
    files.  ``run(n)``: advances n steps; every ``rotorForcePlot`` iterations
    it appends the force rows and writes the sectional files of that
    iteration (steps between written iterations run as one library call).
    The files are byte-compatible with the reference's, so its
    post-processing scripts read them unchanged.
    """

    def __init__(self, case, results_dir, rotor: int = 1):
        self.case = case
        self.dir = Path(results_dir)
        self.rid = f"r{rotor:02d}"
        self.plot = int(case.geti("rotorForcePlot"))
        self.nbc = int(case.geti("nbConvect"))

    def _p(self, name: str) -> Path:
        return self.dir / (self.rid + name)

    def _write_iteration(self, row) -> None:
        it = int(round(row[0]))
        with open(self._p("ForceNonDim.csv"), "a") as f:
            f.write(force_nondim_line(row) + "\n")
        with open(self._p("ForceDim.csv"), "a") as f:
            f.write(force_dim_line(it, self.case.force_dim()) + "\n")
        for b in range(1, self.nbc + 1):
            self._p(f"b{b:02d}ForceDist{it:05d}.csv").write_text(force_dist_text(self.case.force_dist(b)))

    def start(self) -> None:
        self.dir.mkdir(parents=True, exist_ok=True)
        self._p("Params.json").write_text(self.case.params_json())
        if self.plot != 0:
            self._p("ForceDim.csv").write_text(force_dim_header() + "\n")
            self._p("ForceNonDim.csv").write_text(force_nondim_header() + "\n")
            self._p("bladedynamics.csv").write_text(dynamics_header() + "\n")
            self._write_iteration(self.case.ct_hist()[0])

    def step_with_snapshot(self, snapshot):
        """Advances one step through the separate calls and calls
        snapshot(case) between the loads and the wake update, where the
        reference writes its per-step files (filaments2file, probes2file,
        src/main.f90:788,795); writes the force files as run() does.
        Returns (the step's CT row or None on an iteration without loads,
        snapshot's result)."""
        it = int(self.case.geti("iter")) + 1
        self.case.solve_circulation()
        row = self.case.loads() if self.plot > 0 and it % self.plot == 0 else None
        result = snapshot(self.case)
        self.case.wake_step()
        if row is not None:
            self._write_iteration(row)
        return row, result

    def run(self, nsteps: int):
        """Advances nsteps steps; returns their (nsteps, 10) CT rows."""
        out = []
        it = int(self.case.geti("iter"))
        end = it + nsteps
        while it < end:
            k = end - it
            if self.plot > 0:
                k = min(k, self.plot - it % self.plot)  # up to the next written iteration
            rows = self.case.step(k)
            out.append(rows)
            it += k
            if self.plot > 0 and it % self.plot == 0:
                self._write_iteration(rows[-1])
        return np.concatenate(out) if out else np.zeros((0, 10))
