"""Writes tests/golden/reference_kats.json: the known answers of the reference's own tests for this path.

Reads the reference's test sources as text (it cannot be compiled here) and extracts:
  tests/potential/EAM/eam.cpp   E0 (line 119), grad_0 (line 125), perfect-lattice |grad| bound (line 167),
                                the Hessian block H(0,0) of the erased cell and its tolerance (lines 131-141)
  tests/potential/EAM/data.cpp  f_Fe(0), f_Fe(0.02) (lines 42-43)
  tests/neigh/adjacent.cpp      AdjacentCells of a 5^3 grid: interior order, face/edge/corner counts
  tests/system/boxes/hypergrid.cpp  HyperGrid(10, 3).cell_idx at 0, 5, 9.5
Run from the repository root with the REFERENCE environment variable naming the reference's checkout:
    REFERENCE=<path to openFLY> python tests/golden/make_golden.py
"""
from __future__ import annotations

import ast
import json
import os
import re
import sys

REF = os.environ.get("REFERENCE", "")
OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")


def arith(expr: str) -> int:
    """Evaluates an integer expression of + - * and parentheses."""
    tree = ast.parse(expr, mode="eval")
    for node in ast.walk(tree):
        if not isinstance(node, (ast.Expression, ast.BinOp, ast.UnaryOp, ast.Constant, ast.Add, ast.Sub, ast.Mult,
                                 ast.USub)):
            raise ValueError(expr)
    return int(eval(compile(tree, "<kat>", "eval")))


def main() -> None:
    if not REF or not os.path.isdir(REF):
        sys.exit("set REFERENCE to the path of the reference's checkout")
    eam = open(os.path.join(REF, "tests/potential/EAM/eam.cpp")).read()
    data = open(os.path.join(REF, "tests/potential/EAM/data.cpp")).read()
    adj = open(os.path.join(REF, "tests/neigh/adjacent.cpp")).read()
    hyp = open(os.path.join(REF, "tests/system/boxes/hypergrid.cpp")).read()
    kat = {}
    kat["E0"] = float(re.search(r"near\(E0,\s*([-0-9.eE+]+)\)", eam).group(1))
    kat["grad0_component"] = float(re.search(r"Vec::Constant\(([-0-9.eE+]+)\)\)\s*<\s*1e-10", eam).group(1))
    kat["grad0_tol"] = 1e-10
    kat["perfect_grad_norm_max"] = float(re.search(r"gnorm\(cell\[g_\]\)\s*<\s*([-0-9.eE+]+)", eam).group(1))
    block = re.search(r"Mat ngd = Mat\{(.*?)\};", eam, re.S).group(1)
    rows = re.findall(r"\{([^{}]*)\}", block)
    kat["hessian_block_00"] = [[float(v) for v in r.split(",") if v.strip()] for r in rows]
    assert len(kat["hessian_block_00"]) == 3 and all(len(r) == 3 for r in kat["hessian_block_00"])
    kat["hessian_block_tol"] = float(re.search(r"gnorm\(ngd - H\(0, 0\)\)\s*<\s*([-0-9.eE+]+)", eam).group(1))
    fvals = re.findall(r"data\.f\(0\)\.f\(([-0-9.eE+]+)\),\s*([-0-9.eE+]+)\)", data)
    kat["f_Fe"] = [[float(x), float(y)] for x, y in fvals]
    interior = [arith(e) for e in re.findall(r"REQUIRE\(neigh\[\d+\]\s*==\s*([^;]+)\);", adj)]
    kat["adjacent_5cubed"] = {
        "interior_cell": 1 + 1 * 5 + 1 * 5 * 5, "interior": interior,
        "face_cell": 2 + 2 * 5, "face_count": arith(re.search(r"neigh.size\(\) == (9 \+ 8)\)", adj).group(1)),
        "edge_cell": 2, "edge_count": 11, "corner_cell": 0, "corner_count": 7,
    }
    assert len(interior) == 26, len(interior)
    abc = re.findall(r"REQUIRE\(([ABC]) == ([0-9 +*]+)\);", hyp)
    hy = {}
    for name, expr in abc:
        if name not in hy and expr.count("*") == 3:  # the 3-D block
            hy[name] = arith(expr)
    kat["hypergrid_10_rc3"] = {"x": {"A": 0.0, "B": 5.0, "C": 9.5}, "idx": hy}
    kat["sources"] = ["tests/potential/EAM/eam.cpp", "tests/potential/EAM/data.cpp", "tests/neigh/adjacent.cpp",
                      "tests/system/boxes/hypergrid.cpp"]
    json.dump(kat, open(OUT, "w"), indent=1)
    print(json.dumps(kat, indent=1))


if __name__ == "__main__":
    sys.exit(main())
