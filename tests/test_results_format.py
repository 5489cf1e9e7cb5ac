"""The rXXForceNonDim.csv writer reproduces the reference's own files byte for
byte (header and rows of its golden results)."""
import numpy as np

from volcanor_gb300 import results as R


def test_force_nondim_lines_match_the_reference_files(golden_dir, tmp_path):
    for case in ("katzNplotkin-AR04", "elevateTest"):
        ref = (golden_dir / case / "r01ForceNonDim.csv.ref").read_text().splitlines()
        assert ref[0] == R.force_nondim_header()
        rows = []
        for line in ref[1:]:
            vals = line.split()
            rows.append([float(vals[0])] + [float(v) for v in vals[1:]])
            assert R.force_nondim_line(rows[-1]) == line
        out = R.write_force_nondim(tmp_path / f"{case}.csv", np.array(rows))
        assert out.read_text().splitlines() == ref


def test_fortran_e_edge_values():
    assert R.fortran_e(0.0) == "  0.0000000E+00"
    assert R.fortran_e(-1.0) == " -0.1000000E+01"
    assert R.fortran_e(9.9999999e-3) == "  0.1000000E-01"
    assert R.fortran_e(123456.78) == "  0.1234568E+06"
