"""The Julia ccall shim in INTEGRATION.md against the C-ABI structs (CPU only).

Julia passes a struct to ccall by its field layout, so every `struct` of the shim must list the
fields of the C struct (ebgpu.h, mirrored field for field by the ctypes classes in _abi.py) in
the same order with the same types, and every positional constructor call in the shim must give
one value per field (a short call is a MethodError at the first solve)."""
import ctypes as C
import pathlib
import re

import pytest

ROOT = pathlib.Path(__file__).resolve().parents[1]

JULIA_TYPES = {"Int64": C.c_int64, "Int32": C.c_int32, "Float64": C.c_double, "UInt64": C.c_uint64,
               "Cint": C.c_int32, "Cdouble": C.c_double}


def julia_code() -> str:
    text = (ROOT / "INTEGRATION.md").read_text()
    return "\n".join(re.findall(r"```julia\n(.*?)```", text, flags=re.S))


def julia_structs(code: str) -> dict:
    out = {}
    for m in re.finditer(r"\bstruct\s+(\w+)\s*;?(.*?)\bend\b", code, flags=re.S):
        fields = re.findall(r"(\w+)::([\w{}, ]+?)(?=[;\n]|$)", m.group(2))
        out[m.group(1)] = [(n, t.strip()) for n, t in fields]
    return out


def ctype_of(jt: str):
    if jt.startswith("Ptr{"):
        return C.c_void_p
    m = re.fullmatch(r"NTuple\{(\d+),\s*(\w+)\}", jt)
    if m:
        return JULIA_TYPES[m.group(2)] * int(m.group(1))
    return JULIA_TYPES[jt]


def same_type(a, b) -> bool:
    if hasattr(a, "_length_") or hasattr(b, "_length_"):
        return getattr(a, "_length_", None) == getattr(b, "_length_", None) and same_type(a._type_, b._type_)
    if a is C.c_void_p or b is C.c_void_p:
        return C.sizeof(a) == C.sizeof(b) and (a is b or b in (C.c_char_p,) or a in (C.c_char_p,))
    return C.sizeof(a) == C.sizeof(b) and (a in (C.c_double, C.c_float)) == (b in (C.c_double, C.c_float))


def test_shim_structs_match_the_c_abi(eb):
    from earthbox_gb300 import _abi
    structs = julia_structs(julia_code())
    assert {"GridDesc", "SolveOpts", "SolveReport", "HeatParams", "HeatLoopReport", "RecycleParams"} <= set(structs)
    for name, fields in structs.items():
        cls = getattr(_abi, name)
        want = cls._fields_
        assert [f for f, _ in fields] == [f for f, _ in want], name
        for (f, jt), (_, ct) in zip(fields, want):
            assert same_type(ctype_of(jt), ct), (name, f, jt, ct)


def constructor_args(code: str, name: str):
    """Argument counts of every positional call `name(...)` in the shim."""
    counts = []
    for m in re.finditer(rf"(?<![\w.]){name}\(", code):
        depth, i, args, cur = 1, m.end(), 0, ""
        while depth:
            ch = code[i]
            if ch in "([{":
                depth += 1
            elif ch in ")]}":
                depth -= 1
            if depth == 1 and ch == ",":
                args += 1
            elif ch.strip() and depth >= 1:
                cur += ch
            i += 1
        counts.append(args + 1 if cur.strip(")") else 0)
    return counts


@pytest.mark.parametrize("name", ["SolveOpts", "SolveReport", "HeatLoopReport", "GridDesc"])
def test_shim_constructor_calls_fill_every_field(name):
    code = julia_code()
    nfields = len(julia_structs(code)[name])
    calls = constructor_args(code, name)
    assert calls, f"no call of {name} in the shim"
    for n in calls:
        assert n == nfields, f"{name}(...) called with {n} values, the struct has {nfields} fields"
