"""Extract the reference's own known-answer values for the rock-property laws from its test
file (test/tests/rock_props_tests.jl of EarthBox.jl, read as text: Julia is not available here)
into rock_props_reference.json beside this script.  Run in a checkout that has the reference:

    python tests/golden/make_rock_props_reference.py /path/to/EarthBox.jl

The fixture holds the inputs and the expected values of three testsets: the temperature-
dependent heat capacity (TemperatureDependentWaples), and the Liao14 and Sekiguchi-Waples
conductivities."""
import json
import pathlib
import re
import sys


def numbers(block: str) -> list:
    return [float(v.replace("_", "")) for v in re.findall(r"-?[0-9][0-9_]*\.?[0-9]*(?:e-?[0-9]+)?", block)]


def array(text: str, name: str) -> list:
    m = re.search(rf"{name}\s*=\s*\[(.*?)\]", text, flags=re.S)
    body = re.sub(r"#.*", "", m.group(1))
    return numbers(body)


def scalar(text: str, name: str) -> float:
    m = re.search(rf"\b{name}\s*=\s*([-0-9_.e]+)(?:\s*/\s*([-0-9_.e]+))?", text)
    v = float(m.group(1).replace("_", ""))
    return v / float(m.group(2).replace("_", "")) if m.group(2) else v


def kelvin_offset(root: pathlib.Path) -> float:
    """The offset of ConversionFuncs.celsius_to_kelvin (src/utils/ConversionFuncs.jl)."""
    src = (root / "src" / "utils" / "ConversionFuncs.jl").read_text()
    m = re.search(r"function celsius_to_kelvin.*?temperature_celsius\s*\+\s*([0-9.]+)", src, flags=re.S)
    return float(m.group(1))


def main(root: str) -> None:
    src = (pathlib.Path(root) / "test" / "tests" / "rock_props_tests.jl").read_text()
    sets = re.split(r'@testset\s+"', src)[2:]
    cp, liao, sw = sets
    out = {
        "source": "EarthBox.jl test/tests/rock_props_tests.jl (reference known answers, tolerance 1e-9)",
        "celsius_to_kelvin_offset": kelvin_offset(pathlib.Path(root)),
        "waples": {"heat_capacity_at_20celsius": scalar(cp, "heat_capacity_at_20celsius"),
                   "temperatures_celsius": array(cp, "sample_temperatures_celsius"),
                   "expected_cp": array(cp, "expected_cp")},
        "liao14": {"k0": scalar(liao, "k0"), "a": scalar(liao, "a"), "density": scalar(liao, "density"),
                   "gravity": scalar(liao, "gravity"), "depths_m": array(liao, "sample_depths_m"),
                   "gradient_c_per_km": scalar(liao, "temperature_gradient_C_per_km"),
                   "expected_k": array(liao, "expected_k_liao")},
        "sekiguchi_waples": {"k0": scalar(sw, "k0"), "temperatures_celsius": array(sw, "sample_temperatures_celsius"),
                             "expected_k": array(sw, "expected_k_sw")},
    }
    dst = pathlib.Path(__file__).with_name("rock_props_reference.json")
    dst.write_text(json.dumps(out, indent=1) + "\n")
    print(f"wrote {dst}")


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
