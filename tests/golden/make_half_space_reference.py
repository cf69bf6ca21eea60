"""Extract the reference's known answers for half-space cooling from its test file
(test/tests/half_space_cooling_tests.jl of EarthBox.jl, read as text: Julia is not available
here) into half_space_reference.json beside this script, with the unit conversions of
src/utils/ConversionFuncs.jl it uses.  Run in a checkout that has the reference:

    python tests/golden/make_half_space_reference.py /path/to/EarthBox.jl

The same erf law gives the lithosphere temperature of the fracture-zone recycling
(FractureZone.calc_lithosphere_temperature): T = Ta + (Ts - Ta) (1 - erf(z / (2 sqrt(kappa age)))),
age = distance / half spreading rate."""
import json
import pathlib
import re
import sys


def arith(expr: str) -> float:
    """A Julia arithmetic expression of literals, + - * / and parentheses."""
    if not re.fullmatch(r"[0-9.e_+\-*/() ]+", expr):
        raise ValueError(expr)
    return float(eval(expr.replace("_", ""), {"__builtins__": {}}))


def main(root: str) -> None:
    root = pathlib.Path(root)
    conv = (root / "src" / "utils" / "ConversionFuncs.jl").read_text()
    offset = float(re.search(r"function celsius_to_kelvin.*?temperature_celsius\s*\+\s*([0-9.]+)", conv, flags=re.S).group(1))
    factor = arith(re.search(r"function get_factor_cm_yr_to_m_s\(\)::Float64\s*return\s*([^\n]+)", conv).group(1))
    src = (root / "test" / "tests" / "half_space_cooling_tests.jl").read_text()

    def call_arg(name):
        return float(re.search(rf"{name}\s*=\s*[a-z_]+\(([-0-9_.e]+)\)", src).group(1).replace("_", ""))

    def plain(name):
        return float(re.search(rf"{name}\s*=\s*([-0-9_.e]+)", src).group(1).replace("_", ""))

    def array(name):
        body = re.search(rf"{name}\s*=\s*\[(.*?)\]", src, flags=re.S).group(1)
        return [float(v.replace("_", "")) for v in re.findall(r"-?[0-9][0-9_]*\.?[0-9]*(?:e-?[0-9]+)?", body)]

    out = {
        "source": "EarthBox.jl test/tests/half_space_cooling_tests.jl (reference known answers, tolerance 1e-9)",
        "surface_temperature_kelvin": call_arg("surface_temperature_kelvin") + offset,
        "asthenosphere_temperature_kelvin": call_arg("asthenosphere_temperature_kelvin") + offset,
        "distance_from_ridge_meters": plain("distance_from_ridge_meters"),
        "half_spreading_rate_m_s": call_arg("half_spreading_rate_m_s") * factor,
        "thermal_diffusivity_m2_s": plain("thermal_diffusivity_m2_s"),
        "depths_m": array("sample_depths_m"),
        "expected_temperature_kelvin": array("expected_temperature_kelvin"),
    }
    dst = pathlib.Path(__file__).with_name("half_space_reference.json")
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dst}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
