"""Airfoil tables (C81 files, forceCalcSwitch 1) on the CPU: the oracle's
reader and its interpolation (libC81.f90) against an independent numpy
statement -- grid values exactly, bilinear inside a cell, linear along an
axis where the query sits on a grid line (within the single-precision
epsilon), linear extrapolation outside the table, and the continuation
lines of tables with more than 9 Mach numbers."""
import numpy as np
import pytest

from oracle import oracle as O
from volcanor_gb300 import cases as C


def parse(text):
    """The file back into (mach, alpha, [cl, cd, cm]) with numpy."""
    lines = text.splitlines()
    M, N = int(lines[0][30:32]), int(lines[0][32:34])
    k = 1
    tabs = []
    for _ in range(3):
        mach = [float(lines[k][7 + 7 * j:14 + 7 * j]) for j in range(min(9, M))]
        k += 1
        if M > 9:
            mach += [float(lines[k][7 + 7 * j:14 + 7 * j]) for j in range(M - 9)]
            k += 1
        alpha, vals = [], []
        for _i in range(N):
            row = lines[k]
            alpha.append(float(row[:7]))
            v = [float(row[7 + 7 * j:14 + 7 * j]) for j in range(min(9, M))]
            k += 1
            if M > 9:
                v += [float(lines[k][7 + 7 * j:14 + 7 * j]) for j in range(M - 9)]
                k += 1
            vals.append(v)
        tabs.append((np.array(mach), np.array(alpha), np.array(vals)))
    return tabs


def interp(mach, alpha, tab, a, m):
    def iv(x, q):
        n = len(x)
        i = int(np.clip(np.searchsorted(x, q) - 1, 0, n - 2))
        for j in (i, i + 1):
            if abs(x[j] - q) <= np.finfo(np.float32).eps:
                return j, j
        return i, i + 1
    a1, a2 = iv(alpha, a)
    m1, m2 = iv(mach, m)
    if a1 == a2 and m1 == m2:
        return tab[a1, m1]
    if a1 == a2:
        return tab[a1, m1] + (m - mach[m1]) * (tab[a1, m2] - tab[a1, m1]) / (mach[m2] - mach[m1])
    if m1 == m2:
        return tab[a1, m1] + (a - alpha[a1]) * (tab[a2, m1] - tab[a1, m1]) / (alpha[a2] - alpha[a1])
    f = np.array([[tab[a1, m1], tab[a1, m2]], [tab[a2, m1], tab[a2, m2]]])
    return (np.array([alpha[a2] - a, a - alpha[a1]]) @ f @ np.array([mach[m2] - m, m - mach[m1]])
            / (alpha[a2] - alpha[a1]) / (mach[m2] - mach[m1]))


@pytest.mark.parametrize("nmach", [6, 13])
def test_oracle_c81_lookup_against_numpy(tmp_path, nmach):
    text = C.synthetic_airfoil("test section", nmach=nmach)
    f = tmp_path / "sec.C81"
    f.write_text(text)
    tabs = parse(text)
    rng = np.random.default_rng(nmach)
    queries = [(a, m) for a in tabs[0][1][::3] for m in tabs[0][0][::2]]          # grid points
    queries += [(float(a), float(m)) for a, m in zip(rng.uniform(-19, 19, 40), rng.uniform(0.01, 0.74, 40))]
    queries += [(4.0, 0.33), (5.3, tabs[0][0][2]), (-25.0, 0.2), (23.0, 0.9), (6.0 + 1e-8, 0.4)]
    for c in range(3):
        mach, alpha, tab = tabs[c]
        for a, m in queries:
            ref = interp(mach, alpha, tab, a, m)
            got = O.c81_lookup(f, c, a, m)
            assert abs(got - ref) <= 1e-13 * max(1.0, abs(ref)), (c, a, m, got, ref)


def test_c81_writer_layout():
    text = C.synthetic_airfoil("NACA-like", nmach=11)
    lines = text.splitlines()
    assert lines[0][:30].rstrip() == "NACA-like" and lines[0][30:] == "112111211121"
    # 11 Mach numbers: every Mach line and row continues on a second line
    assert len(lines) == 1 + 3 * (2 + 21 * 2)
