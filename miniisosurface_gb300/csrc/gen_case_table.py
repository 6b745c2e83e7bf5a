#!/usr/bin/env python3
"""Generate ``case_table.h``: the marching-cubes triangle case table, packed.

The triangle list of every cube case has to be identical to the one used by
miniIsosurface (``flyingEdges/util/MarchingCubesTables.h:303`` and
``marchingCubes/util/MarchingCubesTables.h:24``), otherwise triangle order and
corner order differ from the reference output.  This script parses that table
from a reference checkout and writes it in a packed form of our own:

    word = (ntri << 60) | sum_t edge_t << (4*t)        t = 0 .. 3*ntri-1

so one 64-bit word per case holds the whole triangle list (at most 5
triangles = 15 edge ids of 4 bits).  ``numTris`` and ``isCut`` are not copied:
they are derived from this word and the cube edge numbering (see
``case_table.h``).

Usage: python gen_case_table.py <path to MarchingCubesTables.h> [out.h]
"""
import re
import os
import sys
from pathlib import Path


def parse_case_triangles(text):
    """Return 256 lists of edge ids (the -1 terminated rows of caseTriangles)."""
    start = text.index("caseTriangles")
    body = text[start:]
    body = body[body.index("{") + 1:]
    rows = re.findall(r"\{([^{}]*)\}", body)[:256]
    cases = []
    for row in rows:
        vals = [int(v) for v in row.replace("\n", " ").split(",") if v.strip()]
        edges = []
        for v in vals:
            if v == -1:
                break
            edges.append(v)
        assert len(edges) % 3 == 0 and len(edges) <= 15
        cases.append(edges)
    assert len(cases) == 256
    return cases


def pack(edges):
    word = (len(edges) // 3) << 60
    for t, e in enumerate(edges):
        assert 0 <= e < 12
        word |= e << (4 * t)
    return word


def render(cases):
    lines = []
    for c in range(0, 256, 4):
        lines.append("    " + ", ".join("0x%016xull" % pack(cases[c + q]) for q in range(4)) + ",")
    return "\n".join(lines)


HEADER = """// Generated by gen_case_table.py -- do not edit.
//
// Marching-cubes triangle cases, one packed 64-bit word per cube case:
//   bits 60..63 : number of triangles (0..5)
//   bits 4t..4t+3 : cube edge id of triangle corner t (t < 3*ntri)
// The triangle lists are the ones of miniIsosurface
// (flyingEdges/util/MarchingCubesTables.h:303), which fixes triangle and
// corner order of the output.  Cube vertex v is bit v of the case id
// (bit set <=> value >= isovalue); vertices v0..v7 sit at
// (i,j,k) (i+1,j,k) (i+1,j+1,k) (i,j+1,k) (i,j,k+1) (i+1,j,k+1) (i+1,j+1,k+1) (i,j+1,k+1).
#pragma once
#include <stdint.h>

#ifdef __CUDACC__
#define ISO_HD __host__ __device__
#else
#define ISO_HD
#endif

static const uint64_t kIsoCaseTris[256] = {
%s
};

// Cube edge e runs from corner kIsoEdgeLo[e] to corner kIsoEdgeHi[e]; the low
// corner always has the smaller grid coordinate along the edge axis.
// e0,e2,e4,e6 are x-edges, e1,e3,e5,e7 y-edges, e8..e11 z-edges.
static const uint8_t kIsoEdgeLo[12] = {0, 1, 3, 0, 4, 5, 7, 4, 0, 1, 3, 2};
static const uint8_t kIsoEdgeHi[12] = {1, 2, 2, 3, 5, 6, 6, 7, 4, 5, 7, 6};

static inline ISO_HD int iso_case_ntris(uint64_t w) { return (int)(w >> 60); }
static inline ISO_HD int iso_case_edge(uint64_t w, int t) { return (int)((w >> (4 * t)) & 15u); }
"""


def main():
    ref = Path(os.environ.get("MINIISO_REFERENCE", "/root/reference"))
    src = Path(sys.argv[1]) if len(sys.argv) > 1 else ref / "flyingEdges" / "util" / "MarchingCubesTables.h"
    out = Path(sys.argv[2]) if len(sys.argv) > 2 else Path(__file__).with_name("case_table.h")
    cases = parse_case_triangles(src.read_text())
    out.write_text(HEADER % render(cases))
    print("wrote", out)


if __name__ == "__main__":
    main()
