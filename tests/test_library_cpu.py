"""CPU-side checks of the product library: it builds for sm_103a, loads, and
exports every entry point include/vlm.h declares (no GPU calls here)."""
import ctypes
import re
from pathlib import Path

import numpy as np
import pytest

from volcanor_gb300 import build as vbuild
from volcanor_gb300 import cases as C
from volcanor_gb300 import lib

ROOT = Path(__file__).resolve().parents[1]


def header_functions():
    text = (ROOT / "include" / "vlm.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(vlm_[a-z0-9_]+)\s*\(", text)))


def test_library_builds_and_exports_every_declared_symbol():
    path = vbuild.build()
    assert path.exists()
    L = ctypes.CDLL(str(path))
    names = header_functions()
    assert "vlm_case_step" in names and "vlm_biot_savart_rings" in names
    for n in names:
        assert hasattr(L, n), f"{n} declared in include/vlm.h but not exported"
    # the Python binding covers the whole ABI
    assert set(names) == set(lib.SIGNATURES), set(names) ^ set(lib.SIGNATURES)


def test_version_and_defaults_without_gpu():
    L = lib.load()
    assert b"sm_103a" in L.vlm_version()
    o = lib.options()
    assert o.precision == lib.PREC_FP64 and o.sum_chunk == 256 and o.near_factor == 4.0
    assert o.solve_mode == -1


def test_error_paths_without_gpu():
    # invalid arguments are rejected on the host before any device work
    L = lib.load()
    assert L.vlm_case_start(None) == 1
    assert L.vlm_case_step(None, 1, None) == 1
    h = ctypes.c_void_p()
    rc = L.vlm_case_create(b"&PARAMS nt = 5 /", b"&PANELS nb = 1 /", b"", None, ctypes.byref(h))
    assert rc != 0 and not h.value


def test_case_text_roundtrip_through_the_oracle_reader():
    from oracle import oracle as O
    c = C.rotor_2blade_hover(nt=12, n_nwake=6, truncate_nt=9)
    s = O.Sim(c.config, c.geom)
    assert s.geti("nb") == 2 and s.geti("ns") == 24 and s.geti("nNwake") == 6 and s.geti("nFwake") == 3
    np.testing.assert_allclose(s.get("dt"), [5.0 * np.pi / 180.0 / 100.0], rtol=1e-15)


def test_fp32_chunk_plan_shapes():
    """The FP32 chunk planner: one chunk when the target blocks alone fill the
    GPU many times, small chunks when a few targets face many rings."""
    big = lib.rings_sum_chunk(1 << 18, 1 << 20, lib.PREC_FP32)
    assert (1 << 18) // 16 <= big <= 1 << 18
    small = lib.rings_sum_chunk(12480, 24, lib.PREC_FP32)
    assert 16 <= small <= 128
    mid = lib.rings_sum_chunk(12480, 13395, lib.PREC_FP32_NEAR64)
    assert 128 <= mid < 12480
    assert lib.rings_sum_chunk(0, 100, lib.PREC_FP32) == 0


def test_binding_arity_matches_header():
    """Every ctypes signature takes as many arguments as include/vlm.h declares."""
    text = (ROOT / "include" / "vlm.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    for name, params in re.findall(r"\b(vlm_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        p = params.strip()
        n = 0 if p in ("", "void") else p.count(",") + 1
        assert len(lib.SIGNATURES[name][1]) == n, (name, n, len(lib.SIGNATURES[name][1]))


def test_options_struct_matches_header():
    """vlm_options field order and types (the Fortran type and ctypes mirror it)."""
    text = (ROOT / "include" / "vlm.h").read_text()
    body = re.search(r"typedef struct vlm_options \{(.*?)\} vlm_options;", text, flags=re.S).group(1)
    body = re.sub(r"/\*.*?\*/", "", body, flags=re.S)
    fields = re.findall(r"\b(int|double)\s+(\w+)\s*;", body)
    mirror = [(("double" if t is ctypes.c_double else "int"), n) for n, t in lib.Options._fields_]
    assert fields == mirror
    integ = (ROOT / "include" / "vlm_gb300.f90").read_text()
    ftype = re.search(r"type, bind\(c\) :: vlm_options(.*?)end type", integ, flags=re.S).group(1)
    fnames = re.findall(r"::\s*(\w+)", ftype)
    assert fnames == [n for _, n in fields]


def test_fortran_interfaces_match_header():
    """The iso_c_binding interfaces shipped for Fortran hosts bind existing
    symbols with the header's argument counts."""
    text = re.sub(r"/\*.*?\*/", "", (ROOT / "include" / "vlm.h").read_text(), flags=re.S)
    arity = {}
    for name, params in re.findall(r"\b(vlm_[a-z0-9_]+)\s*\(([^)]*)\)\s*;", text):
        p = params.strip()
        arity[name] = 0 if p in ("", "void") else p.count(",") + 1
    integ = (ROOT / "include" / "vlm_gb300.f90").read_text().replace("&\n", " ")
    found = re.findall(r"(?:function|subroutine)\s+\w+\(([^)]*)\)\s*bind\(c,\s*name='(vlm_\w+)'\)", integ)
    assert len(found) >= 10
    for args, name in found:
        n = len([a for a in args.split(",") if a.strip()])
        assert arity[name] == n, (name, arity[name], n)


def test_system_argument_checks_without_gpu():
    """vlm_system_create rejects missing rotors and texts on the host."""
    L = lib.load()
    h = ctypes.c_void_p()
    geoms = (ctypes.c_char_p * 1)(b"&PANELS nb = 1 /")
    assert L.vlm_system_create(b"&PARAMS nt = 5 /", 0, geoms, b"", None, ctypes.byref(h)) == 1
    assert L.vlm_system_create(None, 1, geoms, b"", None, ctypes.byref(h)) == 1
    assert not h.value
    assert L.vlm_system_rotor_count(None) == -1
    assert L.vlm_system_start(None) == 1


def test_airfoil_tables_read_on_the_host(tmp_path):
    """A forceCalcSwitch 1 case reads its C81 files when the library builds
    its geometry (vlm_params_json runs that on the host): present files
    load, a missing one is reported, axisymmetry is refused."""
    from volcanor_gb300 import cases as C
    c = C.rotor_2blade_hover(nt=10, n_nwake=4, truncate_nt=6)
    (tmp_path / "a.C81").write_text(C.synthetic_airfoil("a", nmach=11))
    (tmp_path / "b.C81").write_text(C.synthetic_airfoil("b"))
    geo = (c.geom.replace("forceCalcSwitch = 0", "forceCalcSwitch = 1").replace("nAirfoils = 0", "nAirfoils = 2")
           .replace("airfoilSectionLimit = 1.0", "airfoilSectionLimit = 0.6, 1.0")
           .replace("airfoilFile = 0", "airfoilFile = a.C81, b.C81"))
    text = lib.params_json(c.config, geo, tmp_path)
    assert '"forceCalcSwitch"' in text
    with pytest.raises(lib.VlmError):
        lib.params_json(c.config, geo.replace("b.C81", "missing.C81"), tmp_path)
    with pytest.raises(lib.VlmError):
        lib.params_json(c.config, geo.replace("axisymmetrySwitch = 0", "axisymmetrySwitch = 1"), tmp_path)
