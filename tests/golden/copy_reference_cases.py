"""Copy the reference's own 3D JSON cases (and their gmsh meshes) into the test fixtures.

    python tests/golden/copy_reference_cases.py <reference checkout>

(or with the checkout in the DGTD_REFERENCE environment variable). The files are copied
byte for byte from testData/maxwellInputs/[<group>/]<case>/ into
tests/golden/cases/reference/<case>/, so that the tests run the reference's inputs where the
reference checkout is absent.
"""
from __future__ import annotations

import os
import shutil
import sys
from pathlib import Path

HERE = Path(__file__).resolve().parent
CASES = ("3D_PEC", "3D_TFSF", "3D_TFSF_InteriorPEC", "3D_Curved_Element_Test", "3D_SGBC", "3D_Resonant_Cylinder",
         "3D_Resonant_Sphere", "3D_RCS_Sphere_Box_05m_G2",
         "3D_Resonant_Box_TM55/3D_Resonant_Box_TM55_H1_P3",
         "Performance/3D_Resonant_Box_TM55_PERF/3D_Resonant_Box_TM55_H0_P2_PERF",
         "Performance/3D_Resonant_Box_BLEG_TM55_PERF/3D_Resonant_Box_BLEG_TM55_H0_P2_PERF")


def main() -> None:
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DGTD_REFERENCE")
    if not root:
        sys.exit("usage: copy_reference_cases.py <reference checkout>  (or set DGTD_REFERENCE)")
    src = Path(root) / "testData" / "maxwellInputs"
    for entry in CASES:
        name = Path(entry).name
        dst = HERE / "cases" / "reference" / name
        dst.mkdir(parents=True, exist_ok=True)
        for ext in (".json", ".msh"):
            shutil.copyfile(src / entry / f"{name}{ext}", dst / f"{name}{ext}")
            print(f"{src / entry / (name + ext)} -> {dst / (name + ext)}")


if __name__ == "__main__":
    main()
