"""Copy the reference's own full-case fixtures into tests/golden/.

Run once where a checkout of the reference exists, giving its root:

    python tests/golden/make_golden.py <reference checkout>

It copies, unchanged, the inputs (config.nml, geom01.nml, PLOT3D blade file)
and the reference results (referenceResults/*.ref) of the reference's two
integration cases, tests/katzNplotkin-AR04.case and tests/elevateTest.case,
and the inputs of its three tutorial cases (tutorials/*.case: a Caradonna-
Tung rotor, a simple wing, the TR1208 wing from a PLOT3D file).
These are the golden vectors the oracle is pinned to; the GPU machine has no
reference checkout, so the copies travel with the repository.
"""
import shutil
import sys
from pathlib import Path

CASES = {
    "katzNplotkin-AR04": ["config.nml", "geom01.nml"],
    "elevateTest": ["config.nml", "geom01.nml", "elevate.xyz"],
}
# the reference's tutorial cases (inputs only; they ship no results)
TUTORIALS = {
    "caradonna": ["config.nml", "geom01.nml"],
    "simplewing": ["config.nml", "geom01.nml"],
    "tr1208": ["config.nml", "geom01.nml", "TR1208.xyz"],
}


def main(ref_root: str) -> None:
    ref = Path(ref_root)
    out_root = Path(__file__).resolve().parent
    for case, inputs in CASES.items():
        src = ref / "tests" / f"{case}.case"
        dst = out_root / case
        dst.mkdir(parents=True, exist_ok=True)
        for f in inputs:
            shutil.copyfile(src / f, dst / f)
        for f in sorted((src / "referenceResults").glob("*.ref")):
            shutil.copyfile(f, dst / f.name)
        print(f"{case}: {sorted(p.name for p in dst.iterdir())}")
    for case, inputs in TUTORIALS.items():
        src = ref / "tutorials" / f"{case}.case"
        dst = out_root / f"tutorial-{case}"
        dst.mkdir(parents=True, exist_ok=True)
        for f in inputs:
            shutil.copyfile(src / f, dst / f)
        print(f"tutorial-{case}: {sorted(p.name for p in dst.iterdir())}")


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <reference checkout>")
    main(sys.argv[1])
