"""Golden signals of the strong pseudo-periodic form from the CPU oracle
(oracle/strong.py), for the bench's strong leg and tests/test_gpu_strong.py.

Workload: Kuhn box [-8, 8]^3 um, 12 cubes per axis; a z-cylinder of radius 5 um
on whole cubes (compartment 1, periodic staircase); D 3e-3 / 2e-3 um^2/us,
kappa 1e-5 um/us; periodic in x, y, z; PGSE delta 10600 Delta 43100 us, dt 200 us
(270 steps); b 1000 and 3000 s/mm^2 along (1, 0, 0) and (0.6, 0.8, 0).

    python tests/golden/make_strong_fixture.py [out.json]
"""

import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from oracle import strong  # noqa: E402

SETUP = {"box": [-8.0, 8.0], "cubes_per_axis": 12, "radius": 5.0, "D": [3e-3, 2e-3], "kappa": 1e-5,
         "periodic_dir": [1, 1, 1], "delta": 10600.0, "Delta": 43100.0, "dt": 200.0,
         "signals": [{"b": 1000.0, "g": [1.0, 0.0, 0.0]}, {"b": 3000.0, "g": [1.0, 0.0, 0.0]},
                     {"b": 1000.0, "g": [0.6, 0.8, 0.0]}, {"b": 3000.0, "g": [0.6, 0.8, 0.0]}]}


def mesh(setup):
    lo, hi = setup["box"]
    xyz, tets = oracle.box_mesh((lo,) * 3, (hi,) * 3, setup["cubes_per_axis"])
    X = xyz[tets]
    c = 0.5 * (X.min(axis=1) + X.max(axis=1))
    r = setup["radius"]
    reg = (c[:, 0] ** 2 + c[:, 1] ** 2 < r * r).astype(np.int32)
    return xyz, tets, reg


def main(out):
    s = SETUP
    xyz, tets, reg = mesh(s)
    seq = oracle.PGSE(s["delta"], s["Delta"])
    res = []
    for sig in s["signals"]:
        g = np.asarray(sig["g"]) / np.linalg.norm(sig["g"])
        q = oracle.bvalue_to_q(sig["b"], seq.int4gb())
        sd = strong.duplicated_strong(xyz, tets, reg, np.array(s["D"]), 0.0, s["kappa"], s["periodic_dir"], g)
        r = strong.solve_strong(sd, seq, q, s["dt"])
        res.append({"b": sig["b"], "g": sig["g"], "q": q, "signal": r["signal"], "S0": r["S0"],
                    "normalized": r["normalized"], "compartments": r["compartments"], "steps": r["steps"]})
        print(res[-1], flush=True)
    with open(out, "w") as fh:
        json.dump({"setup": s, "n_dofs": int(sd["n"]), "signals": res}, fh, indent=1)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                               "oracle_strong_signals.json"))
