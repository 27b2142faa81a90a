"""Extract the golden values that pin the BioFVM step from the reference's own tests.

Reads the reference's gtest sources as text and writes reference_golden.json next
to this script: for every TEST/TEST_P block, each EXPECT_NEAR / EXPECT_DOUBLE_EQ
assertion (line number, the asserted expression, expected value, tolerance) and
every `std::vector<double> expected = {...}` array.  The tests in tests/ rebuild
each scenario from the cited lines and compare the oracle (and the GPU path)
against these values.

Usage:  python tests/golden/extract_golden.py REFERENCE_ROOT
   or:  PHYSICORE_REFERENCE_ROOT=... python tests/golden/extract_golden.py
(REFERENCE_ROOT is a checkout of the reference project; it is only needed to
regenerate the committed JSON, never at test time.)
"""
from __future__ import annotations

import json
import os
import re
import sys

FILES = [
    "reactions-diffusion/biofvm/kernels/openmp_solver/tests/test_diffusion_solver.cpp",
    "reactions-diffusion/biofvm/kernels/openmp_solver/tests/test_bulk_solver.cpp",
    "reactions-diffusion/biofvm/kernels/openmp_solver/tests/test_dirichlet_solver.cpp",
    "reactions-diffusion/biofvm/kernels/openmp_solver/tests/test_cell_solver.cpp",
]

TEST_RE = re.compile(r"^\s*TEST(?:_P)?\(\s*(\w+)\s*,\s*(\w+)\s*\)")
NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"
NEAR_RE = re.compile(r"EXPECT_NEAR\((.*),\s*(" + NUM + r")\s*,\s*(" + NUM + r")\s*\)\s*;")
DEQ_RE = re.compile(r"EXPECT_DOUBLE_EQ\((.*),\s*(" + NUM + r"|[\w\[\]\.\* +-]+)\s*\)\s*;")


def parse(path: str, rel: str) -> dict:
    out: dict = {}
    cur = None
    lines = open(path, encoding="utf-8").read().splitlines()
    i = 0
    while i < len(lines):
        line = lines[i]
        m = TEST_RE.match(line)
        if m:
            cur = f"{m.group(1)}.{m.group(2)}"
            out[cur] = {"file": rel, "line": i + 1, "asserts": [], "arrays": []}
            i += 1
            continue
        if cur is not None:
            # join continuation lines of a statement
            stmt, j = line, i
            if ("EXPECT_" in line or "expected = {" in line) and ";" not in line:
                while ";" not in stmt and j + 1 < len(lines):
                    j += 1
                    stmt += " " + lines[j].strip()
            m = NEAR_RE.search(stmt)
            if m:
                out[cur]["asserts"].append({"line": i + 1, "kind": "near", "expr": m.group(1).strip(),
                                            "value": float(m.group(2)), "tol": float(m.group(3))})
            else:
                m = DEQ_RE.search(stmt)
                if m:
                    val = m.group(2).strip()
                    try:
                        v = float(val)
                    except ValueError:
                        v = val
                    out[cur]["asserts"].append({"line": i + 1, "kind": "double_eq",
                                                "expr": m.group(1).strip(), "value": v})
            if "expected = {" in stmt:
                body = stmt[stmt.index("{") + 1: stmt.rindex("}")]
                vals = [float(t) for t in re.findall(NUM, body)]
                out[cur]["arrays"].append({"line": i + 1, "values": vals})
            i = j + 1
            continue
        i += 1
    return out


def main() -> None:
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("PHYSICORE_REFERENCE_ROOT")
    if not root:
        sys.exit("usage: extract_golden.py REFERENCE_ROOT (or set PHYSICORE_REFERENCE_ROOT)")
    data = {"source": "bsc-life/PhysiCore reference tests (paths relative to the project root)", "tests": {}}
    for rel in FILES:
        data["tests"].update(parse(os.path.join(root, rel), rel))
    dst = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_golden.json")
    with open(dst, "w", encoding="utf-8") as f:
        json.dump(data, f, indent=1)
    n = sum(len(t["asserts"]) + len(t["arrays"]) for t in data["tests"].values())
    print(f"wrote {dst}: {len(data['tests'])} tests, {n} assertions/arrays")


if __name__ == "__main__":
    main()
