"""Extract the reference's own printed results used to pin the oracle.

Reads the reference notebooks as text (they are outputs of the reference's
solve path run with DOLFIN 2019.1.0) and writes tests/golden/reference_kats.json.
Run where a checkout of the reference exists, giving its root as the argument
or in the environment variable DMRI_REFERENCE:
    python tests/golden/extract_reference_kats.py <reference root>
"""

import json
import os
import re
import sys

LINE = re.compile(r"b: ([0-9.]+), g: ([0-9.]+), q: ([0-9.e+-]+), Signal: ([0-9.e+-]+), "
                  r"Normalized signal: ([0-9.e+-]+), dt: ([0-9.]+), hmin: ([0-9.e+-]+), hmax: ([0-9.e+-]+), "
                  r"whole_vol: ([0-9.]+), vol_of_interest: ([0-9.]+)")


def main(ref):
    nb = json.load(open(os.path.join(ref, "ConvergenceTest.ipynb")))
    found = None
    for cell in nb["cells"]:
        for o in cell.get("outputs", []):
            txt = "".join(o.get("text", []))
            m = LINE.search(txt)
            if m:
                found = m
    keys = ["b", "g", "q", "signal", "normalized", "dt", "hmin", "hmax", "whole_vol", "voi"]
    kat = {k: float(v) for k, v in zip(keys, found.groups())}
    out = {
        "convergence_test_3d_box": {
            "source": "ConvergenceTest.ipynb (printed result of cell 10; setup lines 245, 261-263, "
                      "353, 366-395)",
            "printed": kat,
            "setup": {"box": [-2.5, 2.5], "cubes_per_axis": 16,
                      "why_16": "printed hmin 5.413e-01 = sqrt(3)*5/16 (DOLFIN Cell::h = largest vertex "
                                "distance); the n=5 box in the cell source gives hmin 1.732",
                      "D": 2e-3, "delta": 1000, "Delta": 10000, "dt": 10, "b": 1000, "gdir": [0, 0, 1],
                      "loop": "while t < T (ConvergenceTest.ipynb:374)", "linsolver": "PETScLUSolver mumps"},
            "digits": 7,
        },
        "free_diffusion_b0": {"source": "ExplicitImplementation.ipynb:437", "normalized": 1.0},
    }
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "reference_kats.json")
    json.dump(out, open(path, "w"), indent=1)
    print(json.dumps(out, indent=1))


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMRI_REFERENCE")
    if not root or not os.path.isdir(root):
        sys.exit("give the reference checkout's root as the argument or in DMRI_REFERENCE")
    main(root)
