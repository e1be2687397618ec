"""Extract golden vectors from the reference's own fixtures into small JSON files.

Run with the REFERENCE_ROOT environment variable set to the root of the Iron source tree.  The
JSON files it writes are committed; tests never read the reference tree.

Sources:
  tests/ClassicalField/output_analytic_laplace/AnalyticLaplaceLinearLagrange.opanal
      Iron's analytic-analysis output of the 2D Laplace test (tests/ClassicalField/AnalyticLaplace.F90:
      2x2 bilinear Lagrange elements, origin (-pi/2, -pi/2) with pi = 3.141592653579, extent 2x2,
      u = cos(x) cosh(y) on the boundary (Laplace_equations_routines.F90 TWO_DIM_2), iterative solve
      to 1e-12).  Nodal numerical / analytic values and the integral errors of variable 1.
  tests/ClassicalField/output_analytic_laplace/AnalyticLaplaceLinearSimplex.opanal
      The same test on linear triangles (each grid square split along its (0,0)-(1,1) diagonal,
      generated_mesh_routines.F90:1641-1660; Gauss_Simplex order 3, the default for linear
      triangles, basis_routines.F90:4222-4230).
  tests/ClassicalField/output_analytic_laplace/AnalyticLaplaceCubicHermite.opanal
      The same test on bicubic Hermite elements with 3x3 Gauss points and arithmetic-mean scaling:
      all four derivatives of every node (value, d/ds1, d/ds2, d2/ds1ds2).
  tests/FiniteElasticity/output_cantilever/{linear_3x2x2,cubic_2x1x1}/Cantilever.part0.{exnode,exelem}
      Iron's exported results of the Cantilever finite-elasticity test (FieldExport.c formats):
      copied verbatim into exfile/ to pin the exnode/exelem reader and writer by round trip.
  tests/FiniteElasticity/output_shear/SimpleShear.part0.{exnode,exelem}
      Iron's exported results of the SimpleShear test (triquadratic Lagrange elements of 27 nodes
      with one scale-factor set): copied verbatim into exfile/ as a third round-trip case.
"""
from __future__ import annotations

import json
import os
import re
import shutil
from pathlib import Path

REF = Path(os.environ["REFERENCE_ROOT"]) if os.environ.get("REFERENCE_ROOT") else None
OUT = Path(__file__).resolve().parent


def parse_opanal_variable1(path: Path, setup: dict | None = None) -> dict:
    text = path.read_text()
    block = text.split("Variable 2")[0]
    nodal = block.split("RMS errors")[0]
    nodes = []
    node = None
    # rows "node deriv numerical analytic %err abs rel"; a node's further derivatives omit the node
    for m in re.finditer(r"^\s+(?:(\d+)\s+)?(\d+)\s+(\S+)\s+(\S+)\s+\S+\s+\S+\s+\S+\s*$", nodal, re.M):
        if m.group(1):
            node = int(m.group(1))
        nodes.append({"node": node, "deriv": int(m.group(2)), "numerical": float(m.group(3)),
                      "analytic": float(m.group(4))})
    intg = re.search(r"^\s+1\s+Intg\s+(\S+)\s+(\S+)", block, re.M)
    intg2 = re.search(r"^\s+Intg\^2\s+(\S+)\s+(\S+)", block, re.M)
    return {
        "source": str(path.relative_to(REF)),
        "print_format": "E12.5 (5 significant digits)",
        "nodes": nodes,
        "integral": {"numerical": float(intg.group(1)), "analytic": float(intg.group(2))},
        "integral_sq": {"numerical": float(intg2.group(1)), "analytic": float(intg2.group(2))},
        "setup": setup,
    }


ORIGIN = [-3.141592653579 / 2.0, -3.141592653579 / 2.0]
CASES = {
    "analytic_laplace_linear_lagrange.json": (
        "AnalyticLaplaceLinearLagrange.opanal",
        {"nelem": [2, 2], "basis": "bilinear Lagrange", "gauss": [2, 2], "origin": ORIGIN, "extent": [2.0, 2.0],
         "analytic": "cos(x)*cosh(y)", "dirichlet": "all boundary nodes at analytic values"}),
    "analytic_laplace_linear_simplex.json": (
        "AnalyticLaplaceLinearSimplex.opanal",
        {"nelem": [2, 2], "basis": "linear simplex (triangles, each square split along its (0,0)-(1,1) diagonal)",
         "gauss_simplex_order": 3, "origin": ORIGIN, "extent": [2.0, 2.0], "analytic": "cos(x)*cosh(y)",
         "dirichlet": "all boundary nodes at analytic values"}),
    "analytic_laplace_cubic_hermite.json": (
        "AnalyticLaplaceCubicHermite.opanal",
        {"nelem": [2, 2], "basis": "bicubic Hermite", "gauss": [3, 3], "scaling": "arithmetic mean",
         "origin": ORIGIN, "extent": [2.0, 2.0], "analytic": "cos(x)*cosh(y)",
         "dirichlet": "all four derivatives of all boundary nodes at analytic values"}),
}


def main():
    if REF is None:
        raise SystemExit("set REFERENCE_ROOT to the root of the Iron source tree")
    for name, (fixture, setup) in CASES.items():
        src = REF / "tests/ClassicalField/output_analytic_laplace" / fixture
        data = parse_opanal_variable1(src, setup)
        (OUT / name).write_text(json.dumps(data, indent=1) + "\n")
        print("wrote", OUT / name, len(data["nodes"]), "nodal values")
    (OUT / "exfile").mkdir(exist_ok=True)
    for case in ("linear_3x2x2", "cubic_2x1x1"):
        for ext in ("exnode", "exelem"):
            src = REF / "tests/FiniteElasticity/output_cantilever" / case / f"Cantilever.part0.{ext}"
            dst = OUT / "exfile" / f"cantilever_{case}.{ext}"
            shutil.copyfile(src, dst)
            print("copied", src.relative_to(REF), "->", dst.name)
    for ext in ("exnode", "exelem"):
        src = REF / "tests/FiniteElasticity/output_shear" / f"SimpleShear.part0.{ext}"
        dst = OUT / "exfile" / f"simple_shear.{ext}"
        shutil.copyfile(src, dst)
        print("copied", src.relative_to(REF), "->", dst.name)


if __name__ == "__main__":
    main()
