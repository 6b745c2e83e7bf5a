#!/usr/bin/env python3
"""Generate oracle/case_table.h from a miniIsosurface checkout.

The oracle keeps its own copy of the marching-cubes triangle cases, encoded
as one string of hex digits per case (one digit per triangle corner, i.e. the
cube edge id), so that it does not share a table with the product kernels.
Source: flyingEdges/util/MarchingCubesTables.h:303 (caseTriangles).

Usage: python oracle/gen_case_table.py <path to MarchingCubesTables.h>
"""
import re
import os
import sys
from pathlib import Path


def parse(text):
    body = text[text.index("caseTriangles"):]
    body = body[body.index("{") + 1:]
    rows = re.findall(r"\{([^{}]*)\}", body)[:256]
    out = []
    for row in rows:
        vals = [int(v) for v in row.split(",") if v.strip()]
        out.append("".join("%x" % v for v in vals[: vals.index(-1) if -1 in vals else len(vals)]))
    assert len(out) == 256
    return out


def main():
    ref = Path(os.environ.get("MINIISO_REFERENCE", "/root/reference"))
    src = Path(sys.argv[1]) if len(sys.argv) > 1 else ref / "flyingEdges" / "util" / "MarchingCubesTables.h"
    cases = parse(src.read_text())
    lines = ["// Generated by oracle/gen_case_table.py -- do not edit.",
             "// Test infrastructure: triangle cases of miniIsosurface",
             "// (flyingEdges/util/MarchingCubesTables.h:303) as hex strings, one",
             "// digit per triangle corner (cube edge id), three digits per triangle.",
             "#pragma once",
             "static const char* const kOracleCases[256] = {"]
    for c in range(0, 256, 8):
        lines.append("    " + " ".join('"%s",' % s for s in cases[c:c + 8]))
    lines.append("};")
    out = Path(__file__).with_name("case_table.h")
    out.write_text("\n".join(lines) + "\n")
    print("wrote", out)


if __name__ == "__main__":
    main()
