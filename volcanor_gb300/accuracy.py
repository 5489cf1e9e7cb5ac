"""CT-history accuracy of the reduced-precision solver modes against FP64.

Runs one case in FP64 (the parity mode) and in the FP32 modes, and reports
the relative error of the CT (or CL) history of each mode against FP64 --
per step and averaged over the last revolutions -- next to the FP64 noise
floor: FP64 with a different summation blocking, which differs from the
first FP64 run only by rounding.  A free wake is chaotic (a rounding-level
difference grows until the two wakes are different samples of the same
flow), so the per-step error after many revolutions measures that growth,
and the revolution-averaged CT measures the answer.

    python -m volcanor_gb300.accuracy --case hover2 [--nt 1440] [--out file.npz] [--no-incremental]
"""
import argparse
import json
import tempfile
import time

import numpy as np

from . import cases as C
from . import lib

CASES = {
    "hover2": lambda nt: C.rotor_2blade_hover(nt=nt),
    "forward4": lambda nt: C.rotor_4blade_forward(nt=nt),
    "wing": lambda nt: C.wing_ar4(nt=nt),
}
DEFAULT_NT = {"hover2": 1440, "forward4": 2880, "wing": 200}
STEPS_PER_REV = 72


def run(case_name: str, nt: int, precision: int, sum_chunk=None, chunk_steps: int = 100, incremental=None):
    c = CASES[case_name](nt)
    with tempfile.TemporaryDirectory() as d:
        c.write(d)
        g = lib.Case.from_case_dir(d, precision=precision, sum_chunk=sum_chunk, incremental=incremental)
    g.start()
    rows = []
    t0 = time.perf_counter()
    done = 0
    while done < nt:
        n = min(chunk_steps, nt - done)
        rows.append(g.step(n))
        done += n
    wall = time.perf_counter() - t0
    g.close()
    return np.concatenate(rows), wall


def compare(ref: np.ndarray, x: np.ndarray, avg_steps: int):
    a, b = ref[:, 1], x[:, 1]
    rel = np.abs(b - a) / np.maximum(np.abs(a), 1e-300)
    out = {"max_rel_err": float(rel.max()), "max_rel_err_step": int(np.argmax(rel)) + 1}
    for n in (72, 144, 288):
        if n <= len(rel):
            out[f"max_rel_err_first_{n}"] = float(rel[:n].max())
    if avg_steps <= len(a):
        ma, mb = a[-avg_steps:].mean(), b[-avg_steps:].mean()
        out["avg_window_steps"] = avg_steps
        out["rel_err_of_window_mean"] = float(abs(mb - ma) / abs(ma))
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--case", default="hover2", choices=sorted(CASES))
    ap.add_argument("--nt", type=int, default=None)
    ap.add_argument("--avg-revs", type=int, default=2)
    ap.add_argument("--out", default=None)
    ap.add_argument("--no-floor", action="store_true", help="skip the second FP64 run")
    ap.add_argument("--no-incremental", action="store_true",
                    help="FP32 modes with the full predicted-wake sum (vlm_options.incremental = 0)")
    args = ap.parse_args()
    nt = args.nt or DEFAULT_NT[args.case]
    avg = args.avg_revs * STEPS_PER_REV
    res = {"case": args.case, "nt": nt}
    ref, w = run(args.case, nt, lib.PREC_FP64)
    res["fp64_wall_s"] = round(w, 2)
    hist = {"fp64": ref}
    if not args.no_floor:
        x, w = run(args.case, nt, lib.PREC_FP64, sum_chunk=0)
        hist["fp64_chunk0"] = x
        res["fp64_chunk0"] = compare(ref, x, avg) | {"wall_s": round(w, 2)}
    res["incremental"] = not args.no_incremental
    for name, p in (("fp32near", lib.PREC_FP32_NEAR64), ("fp32", lib.PREC_FP32)):
        x, w = run(args.case, nt, p, incremental=False if args.no_incremental else None)
        hist[name] = x
        res[name] = compare(ref, x, avg) | {"wall_s": round(w, 2)}
    if args.out:
        np.savez_compressed(args.out, **hist)
    print(json.dumps(res))


if __name__ == "__main__":
    main()
