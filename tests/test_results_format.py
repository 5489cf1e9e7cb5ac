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


def test_force_dist_files_round_trip_the_reference_files(golden_dir):
    for case, it in (("katzNplotkin-AR04", 160), ("elevateTest", 1), ("elevateTest", 150)):
        f = golden_dir / case / f"r01b01ForceDist{it:05d}.csv.ref"
        text = f.read_text()
        assert text.splitlines()[0] == "".join(c.rjust(15) for c in R.FORCE_DIST_COLUMNS)
        assert R.force_dist_text(np.loadtxt(f, skiprows=1)) == text


def test_force_dim_and_dynamics_layout():
    # init_plots headers (A5, 11(A15)) and (A5, 5(A15)); force2file rows (A, 11(E15.7))
    assert R.force_dim_header() == "iter" .rjust(5) + "".join(c.rjust(15) for c in R.FORCE_DIM_COLUMNS[1:])
    assert len(R.force_dim_header()) == 5 + 11 * 15
    assert R.dynamics_header() == " iter          pitch           flap          dflap              w          omega"
    line = R.force_dim_line(7, [1.5, 0.0, 0.0, 0.0, 1.5, 0, 0, 0, -2e-3, 0.0, 1.5])
    assert line == "00007" + "  0.1500000E+01  0.0000000E+00" + "  0.0000000E+00" * 2 + "  0.1500000E+01" + \
        "  0.0000000E+00" * 3 + " -0.2000000E-02  0.0000000E+00  0.1500000E+01"


def test_params_json_matches_the_reference_files(golden_dir):
    """rXXParams.json text from the case files (host-side parsing in the
    library, no GPU).  elevateTest's golden file comes from the current
    params2file and matches byte for byte; katzNplotkin-AR04's comes from an
    older key order without the imagePlane / imageRotorNum keys: its lines
    match byte for byte, as a set, once those two lines are dropped."""
    from volcanor_gb300 import lib
    import json
    for case in ("elevateTest", "katzNplotkin-AR04"):
        d = golden_dir / case
        text = lib.params_json((d / "config.nml").read_text(), (d / "geom01.nml").read_text(), d)
        ref = (d / "r01Params.json.ref").read_text()
        if case == "elevateTest":
            assert text == ref
        else:
            kept = [ln for ln in text.splitlines() if '"imagePlane"' not in ln and '"imageRotorNum"' not in ln]
            assert sorted(kept) == sorted(ref.splitlines())
        assert json.loads(text)["nt"] == json.loads(ref)["nt"]


def test_params_json_number_layout():
    """Integers in 12 columns; reals F-form (15 significant digits + 5 blanks)
    for 0.1 <= |x| < 1e15, else E-form with a three-digit exponent."""
    from volcanor_gb300 import cases as C
    from volcanor_gb300 import lib
    cfg = C.config_text(nt=12, dt=0.025, density=1.225, fdScheme=3)
    geo = C.geom_text(nb=1, nc=2, ns=3, nNwake=4, span=2.0, chord=0.5, theta0=-6.5, velBody=(-10.0, 0.0, 0.0))
    lines = {ln.split(":")[0].strip(): ln for ln in lib.params_json(cfg, geo).splitlines() if ":" in ln}
    assert lines['"nt"'] == ' "nt":           12 ,'
    assert lines['"dt"'] == ' "dt":   2.500000000000000E-002 ,'
    assert lines['"density"'] == ' "density":    1.22500000000000      ,'
    assert lines['"theta0"'] == ' "theta0":   -6.50000000000000      ,'
    assert lines['"u"'] == ' "u":   -10.0000000000000      ,'
    assert lines['"radius"'] == ' "radius":    2.00000000000000      ,'
    assert lines['"chord"'] == ' "chord":   0.500000000000000      ,'
