"""Generate the golden fixtures under tests/golden/ from the reference sources.

Run where the reference sources are readable, giving their root directory as the
argument or in the environment variable CRYOIM_REFERENCE:

    python tests/golden/make_golden.py <reference root>

Fixtures written:
  icos2f_sym_mat.json -- the 60 rotation matrices, in file order, parsed from
      icosprocess/SRC/icos2f_sym_mat.f90:5-243 (subroutine icos2f_sym_mat).  They pin
      the operator table and its order (return_icos_asymmetry_unit returns the first
      operator that lands in the asymmetric unit, so the order is observable).
  icos_subgroups.json -- the Cn tables of the same file (c12, c5a, c6, c3, c15, c4, c2,
      c8, c7), evaluated in FP64 from their cos/sin expressions.

The reference ships no test data, so these are the only reference-derived vectors.
"""
from __future__ import annotations

import json
import math
import os
import re
import sys

HERE = os.path.dirname(os.path.abspath(__file__))


def parse_tables(path: str) -> dict[str, list]:
    src = open(path, encoding="latin-1").read()
    parts = re.split(r"\n\s*subroutine\s+(\w+)\s*\(", src, flags=re.I)
    # parts: [pre, name1, body1, name2, body2, ...]; the first subroutine is at file start
    first = re.match(r"\s*subroutine\s+(\w+)\s*\(", parts[0], flags=re.I)
    bodies = {}
    if first:
        bodies[first.group(1).lower()] = parts[0]
    for i in range(1, len(parts), 2):
        bodies[parts[i].lower()] = parts[i + 1]
    out = {}
    assign = re.compile(r"rotmat\(\s*(\d)\s*,\s*(\d)\s*,\s*(\d+)\s*\)\s*=\s*([^;\n]+)", re.I)
    for name, body in bodies.items():
        mats = {}
        for m in assign.finditer(body):
            r, c, k, expr = int(m[1]), int(m[2]), int(m[3]), m[4].strip()
            expr = expr.split("!")[0].strip()
            val = eval(expr.replace("cos(", "math.cos(").replace("sin(", "math.sin(")
                       .replace("sqrt(", "math.sqrt("), {"math": math})
            mats.setdefault(k, [[0.0] * 3 for _ in range(3)])[r - 1][c - 1] = float(val)
        if mats:
            out[name] = [mats[k] for k in sorted(mats)]
    return out


def main(ref: str) -> None:
    tabs = parse_tables(os.path.join(ref, "icosprocess", "SRC", "icos2f_sym_mat.f90"))
    main_tab = tabs.pop("icos2f_sym_mat")
    assert len(main_tab) == 60, len(main_tab)
    src = "icosprocess/SRC/icos2f_sym_mat.f90"
    with open(os.path.join(HERE, "icos2f_sym_mat.json"), "w") as f:
        json.dump({"source": src, "order": "file order (operator 1..60)", "rot": main_tab}, f)
    with open(os.path.join(HERE, "icos_subgroups.json"), "w") as f:
        json.dump({"source": src, "tables": tabs}, f)
    print("wrote", sorted(["icos2f_sym_mat"] + list(tabs)))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("CRYOIM_REFERENCE")
    if not root:
        sys.exit("usage: make_golden.py <reference root>  (or set CRYOIM_REFERENCE)")
    main(root)
