"""Extracts the golden spectral-filter matrices of the reference's own test
(test/Numerics/Mesh/filter.jl, "Exponential and Cutoff filter matrix": hex
Float64 matrices computed with the nodal-dg Filter1D.m, and the filter
arguments they belong to) into filter_matrices.json.

Run from the repository root with the reference checked out:
    python tests/golden/make_filter_golden.py /path/to/ClimateMachine.jl
"""
import json
import os
import re
import struct
import sys


def main(ref_root):
    src = open(os.path.join(ref_root, "test", "Numerics", "Mesh", "filter.jl")).read()
    out = []
    for m in re.finditer(r"W = \[(.*?)\]\s*#! format: on.*?ExponentialFilter\(grid, (\d+), (\d+)\)", src, re.S):
        rows = [r.split() for r in m.group(1).strip().splitlines() if r.strip() and not r.strip().startswith("#")]
        vals = [[struct.unpack(">d", bytes.fromhex(h[2:]))[0] for h in r] for r in rows]
        out.append({"kind": "exponential", "N": len(vals) - 1, "Nc": int(m.group(2)), "s": int(m.group(3)),
                    "W": vals, "source": "test/Numerics/Mesh/filter.jl"})
    if len(out) != 2:
        raise SystemExit(f"expected 2 golden matrices, found {len(out)}")
    with open(os.path.join(os.path.dirname(os.path.abspath(__file__)), "filter_matrices.json"), "w") as f:
        json.dump(out, f, indent=1)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        raise SystemExit("usage: python tests/golden/make_filter_golden.py /path/to/ClimateMachine.jl")
    main(sys.argv[1])
