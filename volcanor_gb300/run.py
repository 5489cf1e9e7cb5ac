"""Run a reference case directory end to end on the GPU: the counterpart of
the reference's main program (src/main.f90) for Python hosts.

Reads the case's ``config.nml`` / ``geom01.nml`` (and PLOT3D files), runs
its ``nt`` timesteps and writes ``Results/`` as the reference does:
``r01Params.json`` at start-up, the force files every ``rotorForcePlot``
iterations (ForceNonDim, ForceDim, bYYForceDistNNNNN) and, every
``gridPlot`` iterations once the far wake exists, ``filamentsNNNNN.dat``,
taken where the reference takes it: inside the iteration, after its loads
and before the wake update (the step's separate calls).  The reference's own
post-processing (tests/test_*.py, parseResults.py) reads the directory
unchanged.

    python -m volcanor_gb300.run <case dir> [--precision fp64|fp32|fp32near] [--steps N]
"""
from __future__ import annotations

import argparse
import sys
import time
from pathlib import Path

from . import gridgen as G
from . import lib
from .results import ResultsWriter

PRECISIONS = {"fp64": lib.PREC_FP64, "fp32": lib.PREC_FP32, "fp32near": lib.PREC_FP32_NEAR64}


def run_case(case_dir, precision: int = lib.PREC_FP64, steps: int | None = None, results_dir=None,
             grid_plot: int | None = None) -> dict:
    """Runs the case in case_dir; returns a summary (steps, wall time, last
    CT row, written filament files)."""
    d = Path(case_dir)
    out = Path(results_dir) if results_dir is not None else d / "Results"
    case = lib.Case.from_case_dir(d, precision=precision)
    t0 = time.perf_counter()
    case.start()
    w = ResultsWriter(case, out)
    w.start()
    nt = case.geti("nt") if steps is None else min(int(steps), case.geti("nt"))
    gp = grid_plot if grid_plot is not None else _grid_plot(d)
    rows, fil = None, []
    it = 0
    def snapshot(c):
        k = c.geti("iter") + 1
        if c.geti("nFwake") > 0 and c.geti("rowFar") <= c.geti("nFwake"):
            return G.write_filaments(out / f"filaments{k:05d}.dat", G.filaments_from_case(c))
        return None

    while it < nt:
        k = nt - it
        if gp > 0:
            k = min(k, gp - it % gp)
        if gp > 0 and (it + k) % gp == 0:
            # the file iteration itself runs as separate calls, the file taken mid-step
            if k > 1:
                rows = w.run(k - 1)
            row, f = w.step_with_snapshot(snapshot)
            if row is not None:
                rows = row[None, :]
            if f is not None:
                fil.append(f)
        else:
            rows = w.run(k)
        it += k
    return {"steps": nt, "wall_s": time.perf_counter() - t0, "last_row": None if rows is None else rows[-1],
            "filament_files": fil}


def _grid_plot(case_dir: Path) -> int:
    """gridPlot of the case, converted as the reference does (from the
    parameters the library echoes into rXXParams.json)."""
    import json
    geo = case_dir / "geom01.nml"
    text = lib.params_json((case_dir / "config.nml").read_text(), geo.read_text(), case_dir)
    return int(json.loads(text)["gridPlot"])


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case_dir")
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default="fp64")
    ap.add_argument("--steps", type=int, default=None, help="stop after this many steps (default: nt)")
    a = ap.parse_args(argv)
    s = run_case(a.case_dir, PRECISIONS[a.precision], a.steps)
    print(f"{s['steps']} steps in {s['wall_s']:.2f} s; last CT row {list(s['last_row'])}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
