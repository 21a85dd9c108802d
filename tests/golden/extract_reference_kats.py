"""Extract the known-answer values of StarFormationHistories.jl's own tests and
doctests into reference_kats.json.

Usage: python extract_reference_kats.py <path of a StarFormationHistories.jl checkout>

Run where a reference checkout exists; the JSON it writes is committed so tests
need no access to the reference at run time.  Each value is read as text from the
file:line recorded beside it.
"""
import json
import os
import re
import sys

if len(sys.argv) != 2:
    raise SystemExit("usage: python extract_reference_kats.py <reference checkout>")
REF = sys.argv[1]
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


def grab(rel, pattern, group=1, cast=float):
    path = os.path.join(REF, rel)
    with open(path) as f:
        lines = f.readlines()
    for i, line in enumerate(lines, 1):
        m = re.search(pattern, line)
        if m:
            return {"value": cast(m.group(group)), "source": f"{rel}:{i}"}
    raise SystemExit(f"pattern {pattern!r} not found in {rel}")


def grab_list(rel, pattern):
    path = os.path.join(REF, rel)
    with open(path) as f:
        lines = f.readlines()
    for i, line in enumerate(lines, 1):
        m = re.search(pattern, line)
        if m:
            vals = [float(v) for v in m.group(1).split(",") if v.strip()]
            return {"value": vals, "source": f"{rel}:{i}"}
    raise SystemExit(f"pattern {pattern!r} not found in {rel}")


kats = {
    "loglikelihood": grab("test/fitting/fitting_core_test.jl",
                          r"loglikelihood\( C, data \) ≈ (-?[0-9.]+)"),
    "loglikelihood_zero_data": grab("test/fitting/fitting_core_test.jl",
                                    r"loglikelihood\( C_zero, data_zero \) ≈ (-?[0-9.]+)"),
    "fg_negative": grab("test/fitting/fitting_core_test.jl", r"-result ≈ (-?[0-9.]+)"),
    "rtol_float32_float64": grab_list("test/fitting/fitting_core_test.jl",
                                      r"const rtols = \(([0-9e.,\- ]+)\)"),
    "gaussian_dispersion_gradient": grab(
        "src/fitting/hierarchical/dispersion_models.jl", r"\(([0-9.]+), -[0-9.]+\)\)"),
    "template_test_mini_spacing_max_diff": grab("test/templates/template_test.jl",
                                                r"maximum\(diff\(result\)\) < ([0-9.]+)"),
}
# The interpolate_mini doctest result spans two lines; read it whole.
with open(os.path.join(REF, "src/StarFormationHistories.jl")) as f:
    txt = f.read()
m = re.search(r"julia> result = \[([^\]]+)\]", txt)
line = txt[: m.start()].count("\n") + 1
kats["interpolate_mini_doctest"] = {
    "value": [float(v) for v in m.group(1).replace("\n", " ").split(",")],
    "source": f"src/StarFormationHistories.jl:{line}"}
json.dump(kats, open(OUT, "w"), indent=1)
print(json.dumps(kats, indent=1))
