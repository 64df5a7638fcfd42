"""Writes tests/golden/mms_functions.py: numpy code of the manufactured
solution and its source (the symbolic derivation of
tests/test_oracle_pins.mms_expressions, for the dry-air gamma of the Earth
constants and mu = 1/100), so that tests can evaluate them where sympy is
not installed.  Run from the repository root:

    python tests/golden/make_mms_functions.py
"""
import os
import sys
from fractions import Fraction

HERE = os.path.dirname(os.path.abspath(__file__))
TESTS = os.path.dirname(HERE)
sys.path.insert(0, TESTS)
sys.path.insert(0, os.path.join(os.path.dirname(TESTS), "oracle"))

import sympy as sp  # noqa: E402
from sympy.printing.numpy import NumPyPrinter  # noqa: E402

import oracle as O  # noqa: E402
from test_oracle_pins import mms_expressions  # noqa: E402


def emit(name, args, exprs, printer):
    repl, red = sp.cse(list(exprs), symbols=sp.numbered_symbols("c"))
    lines = [f"def {name}({', '.join(str(a) for a in args)}):"]
    for sym, e in repl:
        lines.append(f"    {sym} = {printer.doprint(e)}")
    lines.append("    return (" + ", ".join(printer.doprint(e) for e in red) + ",)")
    return "\n".join(lines)


def main():
    c = O.EARTH
    args, q, src = mms_expressions(c["cp_d"] / c["cv_d"], Fraction(1, 100))
    printer = NumPyPrinter({"fully_qualified_modules": True})
    body = "\n\n\n".join([emit("q", args, q, printer), emit("source", args, src, printer)])
    text = ('"""Generated by tests/golden/make_mms_functions.py: the manufactured solution\n'
            "q(t, x, y, z) = (rho, U, V, W, E) of mms_solution.jl and its Navier-Stokes\n"
            'source (gamma = cp_d / cv_d of the Earth constants, mu = 1/100)."""\n'
            "import numpy\n\n\n" + body + "\n")
    with open(os.path.join(HERE, "mms_functions.py"), "w") as f:
        f.write(text)


if __name__ == "__main__":
    main()
