"""Run a reference case directory end to end on the GPU: the counterpart of
the reference's main program (src/main.f90) for Python hosts.

Reads the case's ``config.nml`` / ``geom01.nml`` (and PLOT3D files), runs
its ``nt`` timesteps and writes ``Results/`` as the reference does:
``r01Params.json`` at start-up, the force files every ``rotorForcePlot``
iterations (ForceNonDim, ForceDim, bYYForceDistNNNNN), and the plot files at
the reference's iterations and at its point inside the iteration
(volcanor_gb300.plots): wing and wake geometry (``wakePlot``), wake tip
(``wakeTipPlot``), wake skew (``skewPlotSwitch``), inflow and bound
circulation (``inflowPlotSwitch``, ``gammaPlotSwitch``), filament files for
gridgen (``gridPlot``, once the far wake exists) and probe velocities
(``probe``, from ``probes.in``).  An iteration that writes a file inside
itself runs as the step's separate calls (include/vlm.h), the file taken
between its loads and its wake update; the others run in batches.  The
reference's own post-processing (tests/test_*.py, parseResults.py) reads the
directory unchanged.

A case directory of coupled rotors (``nr > 1`` in config.nml, geom01.nml ..
geomNN.nml, image rotors included) runs as a system (lib.System) and writes
every rotor's ``rXXParams.json`` and force files (ForceNonDim, ForceDim,
bYYForceDistNNNNN) at the reference's iterations; the plot files are
written for single-rotor cases only.

    python -m volcanor_gb300.run <case dir> [--precision fp64|fp32|fp32near] [--steps N]
"""
from __future__ import annotations

import argparse
import re
import sys
import time
from pathlib import Path

from . import gridgen as G
from . import lib
from . import plots as PL
from .results import ResultsWriter

PRECISIONS = {"fp64": lib.PREC_FP64, "fp32": lib.PREC_FP32, "fp32near": lib.PREC_FP32_NEAR64}
SWITCHES = ("wakePlot", "wakeTipPlot", "gridPlot", "probe", "skewPlotSwitch", "inflowPlotSwitch", "gammaPlotSwitch",
            "wakeSuppress", "nNwake")


def _due(sw: dict, k: int) -> dict:
    """The plot files the reference writes inside iteration k."""
    on = lambda n: sw[n] != 0 and k % sw[n] == 0
    wake = sw["wakeSuppress"] == 0 and sw["nNwake"] > 0
    return {"geom": wake and on("wakePlot"), "tip": wake and on("wakeTipPlot"), "skew": wake and on("skewPlotSwitch"),
            "inflow": on("inflowPlotSwitch"), "gamma": on("gammaPlotSwitch"), "fil": on("gridPlot"),
            "probe": on("probe")}


def rotor_count(config_text: str) -> int:
    """nr of a config.nml (1 when absent)."""
    m = re.search(r"^\s*nr\s*=\s*(\d+)", config_text, flags=re.I | re.M)
    return int(m.group(1)) if m else 1


def run_system(case_dir, precision: int = lib.PREC_FP64, steps: int | None = None, results_dir=None,
               sum_chunk: int | None = None) -> dict:
    """Runs a case directory of coupled rotors (nr > 1); writes every rotor's
    Params.json and force files; returns a summary (steps, wall time, the last
    CT row of every rotor)."""
    d = Path(case_dir)
    out = Path(results_dir) if results_dir is not None else d / "Results"
    cfg = (d / "config.nml").read_text()
    nr = rotor_count(cfg)
    geoms = [(d / f"geom{i:02d}.nml").read_text() for i in range(1, nr + 1)]
    y = lib.System(cfg, geoms, d, precision=precision, sum_chunk=sum_chunk)
    t0 = time.perf_counter()
    y.start()
    writers = [ResultsWriter(r, out, rotor=i + 1) for i, r in enumerate(y.rotors)]
    for w in writers:
        w.start()
    nt = y.rotors[0].geti("nt") if steps is None else min(int(steps), y.rotors[0].geti("nt"))
    plot = writers[0].plot
    it, last = 0, None
    while it < nt:
        n = nt - it
        if plot > 0:
            n = min(n, plot - it % plot)  # up to the next written iteration
        rows = y.step(n)
        last = rows[-1]
        it += n
        if plot > 0 and it % plot == 0:
            for ir, w in enumerate(writers):
                w._write_iteration(rows[-1, ir])
    return {"steps": nt, "wall_s": time.perf_counter() - t0, "last_row": last, "rotors": nr}


def run_case(case_dir, precision: int = lib.PREC_FP64, steps: int | None = None, results_dir=None,
             grid_plot: int | None = None, sum_chunk: int | None = None) -> dict:
    """Runs the case in case_dir; returns a summary (steps, wall time, last
    CT row, written plot and filament files).  sum_chunk fixes the
    Biot-Savart summation blocks (lib.Case).  Coupled rotors: run_system."""
    d = Path(case_dir)
    out = Path(results_dir) if results_dir is not None else d / "Results"
    if rotor_count((d / "config.nml").read_text()) > 1:
        return run_system(case_dir, precision, steps, results_dir, sum_chunk)
    cfg, geo = (d / "config.nml").read_text(), (d / "geom01.nml").read_text()
    case = lib.Case(cfg, geo, d, precision=precision, sum_chunk=sum_chunk)
    t0 = time.perf_counter()
    case.start()
    w = ResultsWriter(case, out)
    w.start()
    view = PL.CaseView(case, cfg, geo, d)
    sw = {n: case.geti(n) for n in SWITCHES}
    if grid_plot is not None:
        sw["gridPlot"] = grid_plot
    probes = PL.read_probes(d / "probes.in") if sw["probe"] != 0 else None
    dt, omega, theta0 = case.get("dt")[0], case.get("Omega")[0], case.get("theta0")[0]
    nb = case.geti("nb")
    nt = case.geti("nt") if steps is None else min(int(steps), case.geti("nt"))
    rows, written = None, []
    t = 0.0  # the reference's t: dt added once per iteration
    it = 0

    def step_files(k: int, flags: dict, gam_prev, tk: float):
        def snapshot(c):
            got = []
            ts = f"{k:05d}"
            if flags["skew"]:
                got += PL.skew2file(lambda b: out / f"r01b{b:02d}skew{ts}.csv", view)
            if flags["geom"]:
                got.append(PL.geom2file(out / f"r01wingNwake{ts}.tec", view, k, gam_prev, sw["skewPlotSwitch"] != 0))
            if flags["tip"]:
                got += list(PL.tip2file(out / f"r01tip{ts}.tec", out / f"r01tipXYZ{ts}.csv", view, k, gam_prev,
                                        omega, theta0))
            if flags["inflow"]:
                got += PL.inflow2file(lambda b: out / f"r01b{b:02d}inflowDist{ts}.curve", view)
            if flags["gamma"]:
                got += PL.gamma2file(lambda b: out / f"r01b{b:02d}gammaDist{ts}.curve", view)
            if flags["fil"] and c.geti("nFwake") > 0 and c.geti("rowFar") <= c.geti("nFwake"):
                got.append(G.write_filaments(out / f"filaments{ts}.dat", G.filaments_from_case(c)))
            if flags["probe"] and probes is not None:
                got.append(PL.probes2file(out / f"probes{ts}.csv", view, probes[0], probes[1], tk))
            return got
        return w.step_with_snapshot(snapshot)

    while it < nt:
        # the next iteration that writes a file inside itself
        k = it + 1
        while k <= nt and not any(_due(sw, k).values()):
            k += 1
        if k > it + 1:
            n = min(k, nt + 1) - 1 - it
            r = w.run(n)
            if len(r):
                rows = r
            for _ in range(n):
                t = t + dt
            it += n
            if k > nt:
                break
        gam_prev = [case.get("gam", b) for b in range(1, nb + 1)]
        t = t + dt
        row, got = step_files(k, _due(sw, k), gam_prev, t)
        if row is not None:
            rows = row[None, :]
        written += got
        it = k
    fil = [p for p in written if p.name.startswith("filaments")]
    return {"steps": nt, "wall_s": time.perf_counter() - t0, "last_row": None if rows is None else rows[-1],
            "filament_files": fil, "files": written}


def main(argv=None) -> int:
    ap = argparse.ArgumentParser(description=__doc__.split("\n\n")[0])
    ap.add_argument("case_dir")
    ap.add_argument("--precision", choices=sorted(PRECISIONS), default="fp64")
    ap.add_argument("--steps", type=int, default=None, help="stop after this many steps (default: nt)")
    a = ap.parse_args(argv)
    s = run_case(a.case_dir, PRECISIONS[a.precision], a.steps)
    last = s["last_row"]
    shown = [list(r) for r in last] if last is not None and getattr(last, "ndim", 1) == 2 else list(last)
    print(f"{s['steps']} steps in {s['wall_s']:.2f} s; last CT row {shown}")
    return 0


if __name__ == "__main__":
    sys.exit(main())
