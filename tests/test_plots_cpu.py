"""Plot-file writers on the host (no GPU): the list-directed number layout
against the reference's own golden parameter files, record wrapping, the
probe file reader, the iteration schedule of the plot switches, and the
zone layout of the wing/wake and tip files from a synthetic state."""
from pathlib import Path

import numpy as np
import pytest

from volcanor_gb300 import plots as PL
from volcanor_gb300 import run as RUN

GOLDEN = Path(__file__).parent / "golden"


def _param_items():
    for f in sorted(GOLDEN.glob("*/r01Params.json.ref")):
        for line in f.read_text().splitlines():
            if '": ' not in line or '"' in line.split('": ', 1)[1]:
                continue
            item = line.split('": ', 1)[1]
            item = item[:-2] if item.endswith(" ,") else item
            if "." in item:
                yield f.parent.name, item


def test_ld_real_reproduces_golden_list_directed_reals():
    items = list(_param_items())
    assert len(items) > 40
    for case, item in items:
        assert len(item) == 24, (case, item)
        assert PL.ld_real(float(item.replace("E", "e"))) == item, (case, item)


@pytest.mark.parametrize("x, text", [
    (0.0, "  0.000000000000000E+000"), (1.0, "   1.00000000000000     "), (-0.25, " -0.250000000000000     "),
    (0.1, "  0.100000000000000     "), (0.0999999, "  9.999990000000000E-002"),
    (1e15, "  1.000000000000000E+015"), (123456.789, "   123456.789000000     "),
    (-3.5e-300, " -3.500000000000000E-300"), (float("nan"), "NaN".rjust(24))])
def test_ld_real_ranges(x, text):
    assert len(text) == 24
    assert PL.ld_real(x) == text


def test_ld_lines_three_items_a_record_line():
    s = PL.ld_lines(np.arange(1.0, 8.0))
    lines = s.splitlines()
    assert len(lines) == 3 and all(len(l) <= 80 for l in lines)
    assert [len(l) for l in lines] == [73, 73, 25]
    assert np.array_equal(np.array(" ".join(lines).split(), dtype=float), np.arange(1.0, 8.0))


def test_read_probes(tmp_path):
    (tmp_path / "probes.in").write_text("2\n0.1 0.2 0.3 1.0 0.0 0.0\n-1.0d0, 2.5D-1, 3.0 0.0 -2.0 0.5\n")
    p, v = PL.read_probes(tmp_path / "probes.in")
    np.testing.assert_array_equal(p, [[0.1, 0.2, 0.3], [-1.0, 0.25, 3.0]])
    np.testing.assert_array_equal(v, [[1.0, 0.0, 0.0], [0.0, -2.0, 0.5]])


def test_plot_schedule():
    sw = {"wakePlot": 3, "wakeTipPlot": 0, "gridPlot": 4, "probe": 1, "skewPlotSwitch": 2, "inflowPlotSwitch": 0,
          "gammaPlotSwitch": 5, "wakeSuppress": 0, "nNwake": 4}
    d6 = RUN._due(sw, 6)
    assert d6 == {"geom": True, "tip": False, "skew": True, "inflow": False, "gamma": False, "fil": False,
                  "probe": True}
    assert RUN._due(dict(sw, wakeSuppress=1), 6)["geom"] is False
    assert RUN._due(dict(sw, nNwake=0), 6)["skew"] is False
    assert RUN._due(sw, 20)["fil"] and RUN._due(sw, 20)["gamma"]


class _FakeCase:
    """A two-blade state with a near wake of NW rows (rowNear = 2) and a far
    wake of NF rows (rowFar = 2)."""

    def __init__(self, nc=2, ns=3, NW=4, NF=3):
        rng = np.random.default_rng(0)
        self.i = dict(nb=2, nc=nc, ns=ns, nNwake=NW, nFwake=NF, rowNear=2, rowFar=2, wakeSuppress=0, nbConvect=2,
                      rollupStart=2, rollupEnd=ns)
        self.a = {}
        for b in (1, 2):
            self.a[("gam", b)] = rng.normal(size=nc * ns)
            self.a[("waN", b)] = rng.normal(size=(ns * NW, 4, 3)).ravel()
            self.a[("waN_gam", b)] = -np.abs(rng.normal(size=ns * NW))
            self.a[("waN_age", b)] = np.tile(np.arange(NW, 0, -1) * 0.01, ns)
            self.a[("waF", b)] = rng.normal(size=NF * 6)
            self.a[("waF_gam", b)] = rng.normal(size=NF)
            self.a[("waF_rvc", b)] = np.full(NF, 0.02)
            self.a[("waF_age", b)] = np.arange(NF, 0, -1) * 0.01 + 0.04

    def geti(self, n):
        return self.i[n]

    def get(self, n, b=1):
        if (n, b) not in self.a:
            raise KeyError(n)
        return self.a[(n, b)]


class _FakeView(PL.CaseView):
    def __init__(self, case):
        self.case = case
        self.nb, self.nc, self.ns = 2, case.i["nc"], case.i["ns"]
        self.NW, self.NF = case.i["nNwake"], case.i["nFwake"]

    def panel_corners(self, k, b):
        return np.arange(self.nc * self.ns * 12, dtype=float).reshape(-1, 4, 3) * (b + k)


def _zones(text):
    return [l.strip() for l in text.splitlines() if l.strip().startswith("Zone")]


def test_geom_and_tip_file_layout(tmp_path):
    c = _FakeCase()
    v = _FakeView(c)
    gam_prev = [c.get("gam", b) for b in (1, 2)]
    t = PL.geom2file(tmp_path / "g.tec", v, 3, gam_prev, True).read_text()
    assert _zones(t) == ['Zone I=3 J=4 K=1  T="Blade 01"', 'Zone I=4 J=4 K=1  T="NearWake"',
                         'Zone I=3 J=1   K=1   T="FarWake"', 'Zone I=2 J=1   K=1   T="PrescFarWake"'] + \
                        ['Zone I=3 J=4 K=1  T="Blade 02"', 'Zone I=4 J=4 K=1  T="NearWake"',
                         'Zone I=3 J=1   K=1   T="FarWake"', 'Zone I=2 J=1   K=1   T="PrescFarWake"']
    # blade zone: 3 x (3 x 4) nodes, then 6 gam and 6 zeros (cell centred)
    first = t.split('T="Blade 01"')[1].split("Zone")[0].splitlines()[3:]
    vals = np.array(" ".join(first).split(), dtype=float)
    assert vals.size == 3 * 12 + 2 * 6
    np.testing.assert_allclose(vals[36:42], -1.0 * gam_prev[0], rtol=1e-14)  # 15 significant digits
    tec, csv = PL.tip2file(tmp_path / "t.tec", tmp_path / "t.csv", v, 3, gam_prev, 100.0, 0.1)
    assert _zones(tec.read_text()) == ['Zone I=3 J=4 K=1  T="Blade"', 'Zone I=4 J=1    K=1  T="NearWake"',
                                       'Zone I=3 J=1   K=1   T="FarWake"'] * 2
    rows = [l for l in csv.read_text().splitlines() if "X" not in l]
    assert len(rows) == 2 * ((4 - 1 + 1) + (3 - 1 + 1))
    # roll-up centroid of the first written row: circulation-weighted corner 4 of stations rollupStart..ns
    wn = c.get("waN", 1).reshape(3, 4, 4, 3)
    wg = c.get("waN_gam", 1).reshape(3, 4)
    ref = sum(wn[j, 1, 3] * wg[j, 1] for j in (1, 2)) / (wg[1, 1] + wg[2, 1])
    np.testing.assert_allclose(np.array(rows[0].split(), dtype=float), ref, rtol=1e-14)


def test_skew_file_rows_oldest_first(tmp_path):
    c = _FakeCase()
    v = _FakeView(c)
    files = PL.skew2file(lambda b: tmp_path / f"s{b}.csv", v)
    lines = files[0].read_text().splitlines()
    assert lines[0] == "            max            avg" and len(lines) == 1 + 3
    sk = v.wake_skew(1)
    assert np.all((sk >= 0) & (sk <= 1))
    np.testing.assert_allclose(float(lines[1].split()[0]), sk[:, 3].max(), rtol=1e-6)
