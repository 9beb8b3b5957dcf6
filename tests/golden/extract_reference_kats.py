"""Extract the reference's element-matrix known-answer values into a JSON fixture.

Reads the reference's own GoogleTest sources (Hesthaven & Warburton comparison
tests) and writes ``reference_kats.json`` beside this script. Run it where the
reference checkout is available:

    python tests/golden/extract_reference_kats.py <reference checkout>

(or with the checkout in the DGTD_REFERENCE environment variable).

Only numeric literals are taken (the expected matrices of each test); the
fixture records the source file and line of every matrix.
"""
from __future__ import annotations

import json
import re
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent

# (key, relative file, variable name, occurrence index, scale applied by the test)
WANTED = [
    ("1d_mass_o1", "test/hesthavenComparison/Hesthaven1DTest.cpp", "expected", 0),
    ("1d_invmass_o1", "test/hesthavenComparison/Hesthaven1DTest.cpp", "expected", 1),
    ("1d_stiffness_o1", "test/hesthavenComparison/Hesthaven1DTest.cpp", "expected", 2),
    ("1d_D_o1", "test/hesthavenComparison/Hesthaven1DTest.cpp", "expected", 3),
    ("1d_D_o2", "test/hesthavenComparison/Hesthaven1DTest.cpp", "expected", 4),
    ("1d_D_o4", "test/hesthavenComparison/Hesthaven1DTest.cpp", "expected", 5),
    ("1d_MS_3E", "test/hesthavenComparison/Hesthaven1DTest.cpp", "MS_Hesthaven3E", 0),
    ("1d_MF_4E", "test/hesthavenComparison/Hesthaven1DTest.cpp", "MF_Hesthaven4E", 0),
    ("1d_MF_3E", "test/hesthavenComparison/Hesthaven1DTest.cpp", "MF_Hesthaven3E", 0),
    ("1d_MS4E_block", "test/hesthavenComparison/HesthavenFunctions.cpp", "blockMat", 1),
    ("3d_mass_o2_vvt_inv", "test/hesthavenComparison/Hesthaven3DTest.cpp", "vanderProdInverse", 0),
    ("3d_Dr_o1", "test/hesthavenComparison/Hesthaven3DTest.cpp", "DrOperatorHesthaven", 0),
    ("3d_Ds_o1", "test/hesthavenComparison/Hesthaven3DTest.cpp", "DsOperatorHesthaven", 0),
    ("3d_Dt_o1", "test/hesthavenComparison/Hesthaven3DTest.cpp", "DtOperatorHesthaven", 0),
    ("3d_rotator_o1", "test/hesthavenComparison/Hesthaven3DTest.cpp", "rotatorO1_", 0),
    ("3d_emat_o1", "test/hesthavenComparison/Hesthaven3DTest.cpp", "expected_emat", 0),
]

NUM = r"[-+]?(?:\d+\.?\d*|\.\d+)(?:[eE][-+]?\d+)?"


def _matrix_after(text: str, name: str, occurrence: int):
    # "<name>{" or "<name> {" or "<name> = ...{" followed by a braced list of braced rows
    pat = re.compile(r"\b" + re.escape(name) + r"\s*(?:=\s*[\w:<>, ]*)?\{")
    hits = list(pat.finditer(text))
    if len(hits) <= occurrence:
        raise KeyError(f"{name} #{occurrence} not found")
    m = hits[occurrence]
    i = m.end()
    depth, j = 1, i
    while depth and j < len(text):
        if text[j] == "{":
            depth += 1
        elif text[j] == "}":
            depth -= 1
        j += 1
    body = text[i:j - 1]
    rows = re.findall(r"\{([^{}]*)\}", body)
    mat = []
    for r in rows:
        vals = []
        for item in r.split(","):
            item = item.strip()
            if not item:
                continue
            if not re.fullmatch(r"[-+*/ .\deE]+", item):
                raise ValueError(f"non-numeric entry {item!r} in {name}")
            vals.append(float(eval(item, {"__builtins__": {}}, {})))   # literals like 2.0 / 6.0
        mat.append(vals)
    line = text.count("\n", 0, m.start()) + 1
    return mat, line


def extract(ref_root: Path) -> dict:
    out = {}
    for key, rel, name, occ in WANTED:
        text = (ref_root / rel).read_text()
        mat, line = _matrix_after(text, name, occ)
        out[key] = {"source": f"{rel}:{line}", "matrix": mat}
    return out


def main() -> None:
    import os
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DGTD_REFERENCE")
    if not root:
        sys.exit("usage: extract_reference_kats.py <reference checkout>  (or set DGTD_REFERENCE)")
    ref = Path(root)
    data = extract(ref)
    (HERE / "reference_kats.json").write_text(json.dumps(data, indent=1))
    print(f"wrote {len(data)} matrices to {HERE / 'reference_kats.json'}")


if __name__ == "__main__":
    main()
