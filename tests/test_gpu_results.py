"""The Results/ outputs beside the CT history: sectional loads
(rXXbYYForceDistNNNNN.csv), rotor forces (rXXForceDim.csv) and the case
parameters (rXXParams.json), from the GPU solver.

The sectional and rotor values are compared with the oracle bit for bit; a
whole Results/ directory written by ResultsWriter is then read back the way
the reference's own integration tests read theirs
(tests/test_katzNplotkinAR04.py, tests/test_elevate.py) and checked against
the reference's golden files with the same places=6 tolerance.
"""
import json

import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib
from volcanor_gb300 import results as R

pytestmark = pytest.mark.gpu


def both(cfg, geo, base="", chunk=16):
    g = lib.Case(cfg, geo, base, precision=lib.PREC_FP64, sum_chunk=chunk)
    r = O.Sim(cfg, geo, base)
    r.set_sum_chunk(chunk)
    g.start()
    r.start()
    return g, r


def assert_outputs_equal(g, r, nbc):
    for b in range(1, nbc + 1):
        np.testing.assert_array_equal(g.force_dist(b), r.get("forceDist", b).reshape(-1, 16))
    ref_dim = np.r_[0, 0, r.get("rotorLift"), 0, 0, 0, r.get("rotorForceInertial")]
    ref_dim[0] = np.sqrt(np.sum(ref_dim[2:5] ** 2))
    np.testing.assert_array_equal(g.force_dim()[2:], ref_dim[2:])
    assert g.force_dim()[0] == pytest.approx(ref_dim[0], rel=1e-15)


@pytest.mark.parametrize("fd", [1, 3])
def test_sectional_and_rotor_loads_bitwise_wing(fd):
    cfg = C.config_text(nt=12, dt=0.025, density=1.0, fdScheme=fd)
    geo = C.geom_text(nb=1, nc=3, ns=5, nNwake=6, span=2.0, chord=0.5, theta0=6.0, velBody=(-10.0, 0.0, 0.0),
                      wakeTruncateNt=10)
    g, r = both(cfg, geo)
    assert_outputs_equal(g, r, 1)  # iteration 0 (the initial solve)
    for _ in range(3):
        g.step(4)
        r.step(4)
        assert_outputs_equal(g, r, 1)


def test_sectional_and_rotor_loads_bitwise_rotor():
    c = C.rotor_2blade_hover(nt=30, n_nwake=10, truncate_nt=20)
    g, r = both(c.config, c.geom, chunk=64)
    g.step(30)
    r.step(30)
    assert_outputs_equal(g, r, 2)


def test_sectional_loads_bitwise_axisymmetric_plot3d(golden_dir):
    """elevateTest: 5 blades, axisymmetry (one convected blade), PLOT3D geometry."""
    d = golden_dir / "elevateTest"
    g, r = both((d / "config.nml").read_text(), (d / "geom01.nml").read_text(), base=d, chunk=256)
    assert g.geti("nbConvect") == 1
    g.step(40)
    r.step(40)
    assert_outputs_equal(g, r, 1)


def test_params_json_of_a_case_matches_host_text(golden_dir):
    d = golden_dir / "elevateTest"
    cfg, geo = (d / "config.nml").read_text(), (d / "geom01.nml").read_text()
    g = lib.Case(cfg, geo, d, precision=lib.PREC_FP64)
    assert g.params_json() == lib.params_json(cfg, geo, d) == (d / "r01Params.json.ref").read_text()


@pytest.mark.parametrize("case,nt,written", [("katzNplotkin-AR04", 160, 160), ("elevateTest", 150, 150)])
def test_results_directory_reads_like_the_reference(golden_dir, tmp_path, case, nt, written):
    """Writes Results/ through ResultsWriter and applies the checks of the
    reference's tests/test_katzNplotkinAR04.py and tests/test_elevate.py."""
    d = golden_dir / case
    g = lib.Case.from_case_dir(d, precision=lib.PREC_FP64, sum_chunk=256)
    g.start()
    w = R.ResultsWriter(g, tmp_path)
    w.start()
    rows = w.run(nt)
    assert rows.shape == (nt, 10)
    # testParams
    params = json.loads((tmp_path / "r01Params.json").read_text())
    params_ref = json.loads((d / "r01Params.json.ref").read_text())
    for k, v in params_ref.items():
        if isinstance(v, float):
            assert params[k] == pytest.approx(v, abs=5e-7), k
        else:
            assert params[k] == v, k
    # testCT
    hist = np.loadtxt(tmp_path / "r01ForceNonDim.csv", skiprows=1)
    ref = np.loadtxt(d / "r01ForceNonDim.csv.ref", skiprows=1)
    assert hist.shape == ref.shape
    assert abs(hist[-1, 1] - ref[-1, 1]) < 5e-7
    assert abs(hist[-10:, 1].mean() - ref[-10:, 1].mean()) < 5e-7
    # testSect: the latest sectional file, five columns; both files print 7
    # significant digits, so one unit of the seventh digit (a rounding flip
    # of values that agree to ~1e-13) is allowed beside places=6
    last = sorted(tmp_path.glob("r01b01ForceDist*.csv"))[-1]
    assert last.name == f"r01b01ForceDist{written:05d}.csv"
    names = last.read_text().split("\n", 1)[0].split()
    data = np.loadtxt(last, skiprows=1)
    data_ref = np.loadtxt(d / f"r01b01ForceDist{written:05d}.csv.ref", skiprows=1)
    for col in ("secSpan", "secCL", "secArea", "secVel", "secAlpha"):
        j = names.index(col)
        np.testing.assert_allclose(data[:, j], data_ref[:, j], rtol=1.01e-6, atol=5e-7, err_msg=col)
    # one sectional file per written iteration, one ForceDim row per written iteration
    assert len(list(tmp_path.glob("r01b01ForceDist*.csv"))) == nt + 1
    dim = np.loadtxt(tmp_path / "r01ForceDim.csv", skiprows=1)
    assert dim.shape == (nt + 1, 12)
    np.testing.assert_allclose(dim[:, 9:12] / g.get("nonDimDenom")[0], hist[:, 7:10], rtol=2e-6, atol=1e-12)
