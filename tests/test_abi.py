"""The C-ABI library loads and exports every symbol include/ebgpu.h declares (no GPU calls)."""
import pathlib
import re

import numpy as np

ROOT = pathlib.Path(__file__).resolve().parents[1]


def header_functions():
    text = (ROOT / "include" / "ebgpu.h").read_text()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(eb_[a-z0-9_]+)\s*\(", text)))


def test_library_exports_header_symbols(eb):
    eb.build()
    from earthbox_gb300 import _abi
    lib = _abi.load()
    names = header_functions()
    assert len(names) >= 30
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(_abi.ALL_SYMBOLS) <= set(names)


def test_field_tables_match_header(eb):
    from earthbox_gb300 import _abi
    text = (ROOT / "include" / "ebgpu.h").read_text()
    m_enum = re.search(r"enum eb_marker_field \{(.*?)\};", text, re.S).group(1)
    g_enum = re.search(r"enum eb_grid_field \{(.*?)\};", text, re.S).group(1)
    m_names = re.findall(r"EB_M_([A-Z0-9_]+)", re.sub(r"/\*.*?\*/", "", m_enum, flags=re.S))
    g_names = re.findall(r"EB_G_([A-Z0-9_]+)", re.sub(r"/\*.*?\*/", "", g_enum, flags=re.S))
    assert m_names[-1] == "NFIELDS" and g_names[-1] == "NFIELDS"
    assert len(m_names) - 1 == len(_abi.MARKER_FIELDS)
    assert len(g_names) - 1 == len(_abi.GRID_FIELDS)


def test_grid_shapes(eb):
    from earthbox_gb300 import _abi
    X, Y = 7, 5
    assert _abi.grid_shape("rho1", X, Y) == (Y, X)
    assert _abi.grid_shape("etan1", X, Y) == (Y - 1, X - 1)
    assert _abi.grid_shape("pr1", X, Y) == (Y - 1, X - 1)
    assert _abi.grid_shape("vx1", X, Y) == (Y + 1, X)
    assert _abi.grid_shape("vy1", X, Y) == (Y, X + 1)
    assert _abi.grid_shape("btopt", X, Y) == (X, 2)
    assert _abi.grid_shape("bleftt", X, Y) == (Y, 2)


def test_synthetic_layout_follows_reference_order(eb):
    m = eb.synthetic.config("sinking_block")
    assert m.marknum == 160_000
    # MarkersRandomized: x outer loop, y inner loop -> y cycles fastest
    my = (m.grid.ynum - 1) * 4
    assert np.all(np.diff(m.markers["y"][:my]) > 0)
    assert m.markers["x"][my] > m.markers["x"][0]
    g = m.grid
    assert len(g.gridx_vy) == g.xnum + 1 and len(g.xstp_vy) == g.xnum
    assert np.allclose(g.gridx_vy[1:-1], 0.5 * (g.gridx_b[1:] + g.gridx_b[:-1]))
