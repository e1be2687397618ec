"""Extract golden vectors from the reference's own fixtures into small JSON files.

Run in a container where the reference tree is mounted (default /root/reference, or the
REFERENCE_ROOT environment variable).  The JSON files it writes are committed; tests never read
the reference tree.

Sources:
  tests/ClassicalField/output_analytic_laplace/AnalyticLaplaceLinearLagrange.opanal
      Iron's analytic-analysis output of the 2D Laplace test (tests/ClassicalField/AnalyticLaplace.F90:
      2x2 bilinear Lagrange elements, origin (-pi/2, -pi/2) with pi = 3.141592653579, extent 2x2,
      u = cos(x) cosh(y) on the boundary (Laplace_equations_routines.F90 TWO_DIM_2), iterative solve
      to 1e-12).  Nodal numerical / analytic values and the integral errors of variable 1.
  tests/FiniteElasticity/output_cantilever/{linear_3x2x2,cubic_2x1x1}/Cantilever.part0.{exnode,exelem}
      Iron's exported results of the Cantilever finite-elasticity test (FieldExport.c formats):
      copied verbatim into exfile/ to pin the exnode/exelem reader and writer by round trip.
"""
from __future__ import annotations

import json
import os
import re
import shutil
from pathlib import Path

REF = Path(os.environ.get("REFERENCE_ROOT", "/root/reference"))
OUT = Path(__file__).resolve().parent


def parse_opanal_variable1(path: Path) -> dict:
    text = path.read_text()
    block = text.split("Variable 2")[0]
    nodes = []
    for m in re.finditer(r"^\s+(\d+)\s+1\s+(\S+)\s+(\S+)\s+\S+\s+\S+\s+\S+\s*$", block, re.M):
        nodes.append({"node": int(m.group(1)), "numerical": float(m.group(2)), "analytic": float(m.group(3))})
    intg = re.search(r"^\s+1\s+Intg\s+(\S+)\s+(\S+)", block, re.M)
    intg2 = re.search(r"^\s+Intg\^2\s+(\S+)\s+(\S+)", block, re.M)
    return {
        "source": str(path.relative_to(REF)),
        "print_format": "E12.5 (5 significant digits)",
        "nodes": nodes,
        "integral": {"numerical": float(intg.group(1)), "analytic": float(intg.group(2))},
        "integral_sq": {"numerical": float(intg2.group(1)), "analytic": float(intg2.group(2))},
        "setup": {"nelem": [2, 2], "basis": "bilinear Lagrange", "gauss": [2, 2],
                  "origin": [-3.141592653579 / 2.0, -3.141592653579 / 2.0], "extent": [2.0, 2.0],
                  "analytic": "cos(x)*cosh(y)", "dirichlet": "all boundary nodes at analytic values"},
    }


def main():
    src = REF / "tests/ClassicalField/output_analytic_laplace/AnalyticLaplaceLinearLagrange.opanal"
    data = parse_opanal_variable1(src)
    (OUT / "analytic_laplace_linear_lagrange.json").write_text(json.dumps(data, indent=1) + "\n")
    print("wrote", OUT / "analytic_laplace_linear_lagrange.json", len(data["nodes"]), "nodes")
    (OUT / "exfile").mkdir(exist_ok=True)
    for case in ("linear_3x2x2", "cubic_2x1x1"):
        for ext in ("exnode", "exelem"):
            src = REF / "tests/FiniteElasticity/output_cantilever" / case / f"Cantilever.part0.{ext}"
            dst = OUT / "exfile" / f"cantilever_{case}.{ext}"
            shutil.copyfile(src, dst)
            print("copied", src.relative_to(REF), "->", dst.name)


if __name__ == "__main__":
    main()
