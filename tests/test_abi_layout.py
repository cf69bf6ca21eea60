"""Every ctypes mirror of a C-ABI struct has the header's layout: the same size and each field at
the header's offset (gcc compiles a probe against include/ebgpu.h; a field the header lacks fails
the compile)."""
import ctypes as C
import pathlib
import shutil
import subprocess

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]

PAIRS = {
    "GridDesc": "eb_grid_desc", "MaterialDesc": "eb_material_desc", "Params": "eb_params",
    "StokesParams": "eb_stokes_params", "SolveOpts": "eb_solve_opts", "SolveReport": "eb_solve_report",
    "StokesNorms": "eb_stokes_norms", "MobileWall": "eb_mobile_wall", "LearnedOpts": "eb_learned_opts",
    "LearnedReport": "eb_learned_report", "MarkerIO": "eb_marker_io", "RockDesc": "eb_rock_desc",
    "SedimentDesc": "eb_sediment_desc", "RockParams": "eb_rock_params", "RecycleParams": "eb_recycle_params",
    "HeatParams": "eb_heat_params", "HeatLoopReport": "eb_heat_loop_report",
}


def test_ctypes_structs_match_the_header(eb, tmp_path):
    if shutil.which("gcc") is None:
        pytest.skip("gcc not available")
    abi = eb._abi
    lines = ["#include <stdio.h>", "#include <stddef.h>", '#include "ebgpu.h"', "int main(void) {"]
    want = {}
    for py, c in PAIRS.items():
        cls = getattr(abi, py)
        lines.append(f'  printf("{py} size %zu\\n", sizeof({c}));')
        want[(py, "size")] = C.sizeof(cls)
        for name, _ in cls._fields_:
            lines.append(f'  printf("{py} {name} %zu\\n", offsetof({c}, {name}));')
            want[(py, name)] = getattr(cls, name).offset
    lines += ["  return 0;", "}"]
    src = tmp_path / "probe.c"
    src.write_text("\n".join(lines) + "\n")
    exe = tmp_path / "probe"
    r = subprocess.run(["gcc", "-std=c99", "-I", str(ROOT / "include"), str(src), "-o", str(exe)],
                       capture_output=True, text=True)
    assert r.returncode == 0, r.stderr[-2000:]
    out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split("\n")
    got = {}
    for ln in out:
        if ln.strip():
            py, name, val = ln.split()
            got[(py, name)] = int(val)
    bad = {k: (got.get(k), v) for k, v in want.items() if got.get(k) != v}
    assert not bad, bad
