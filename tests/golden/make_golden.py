"""Generate the oracle golden fixtures used by the GPU parity tests.

Run from the repository root:  python tests/golden/make_golden.py
Writes tests/golden/oracle_signals.json.  Every entry is the FP64 oracle
(``oracle.solve_duplicated`` with the reference's MUMPS-LU alternative, here
SuperLU) on a seeded workload from ``meshgen.workload``; the GPU tests rebuild
the same mesh from the same seed and compare signals.  The oracle itself is
pinned by tests/test_oracle_pins.py against the reference's printed results.
"""

import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

pkg = importlib.import_module("dmri-fem-cloud_gb300")


def oracle_profile(p):
    if p.name == "PGSE":
        return oracle.PGSE(10600, 43100)
    if p.name == "cos-OGSE":
        return oracle.CosOGSE(10600, 43100)
    raise ValueError(p.name)


def run_case(name, n=None, pick=None, seed=0):
    w = pkg.meshgen.workload(name, seed=seed, n=n)
    D = np.asarray(w["D"], np.float64)
    iT2 = 0.0 if w["invT2"] is None else np.asarray(w["invT2"], np.float64)
    kap = 0.0 if w["kappa"] is None else w["kappa"]
    field = None if w["multiple"] else np.zeros(len(w["tets"]), np.int64)
    sd = oracle.duplicated_system(w["xyz"], w["tets"], w["region"], D, iT2, kap, field=field)
    sigs = w["signals"] if pick is None else [w["signals"][i] for i in pick]
    idx = list(range(len(w["signals"]))) if pick is None else list(pick)
    out = []
    for i, (b, g, pi) in zip(idx, sigs):
        prof = oracle_profile(w["profiles"][pi])
        q = oracle.bvalue_to_q(b, prof.int4gb())
        t0 = time.time()
        r = oracle.solve_duplicated(sd, prof, q, g, w["dt"])
        out.append({"index": i, "b": b, "gdir": list(g), "profile": pi, "q": q,
                    "signal": r.signal, "S0": r.S0, "normalized": r.normalized,
                    "compartments": r.compartment_signals, "steps": r.steps,
                    "oracle_seconds": time.time() - t0})
        print(name, n, i, "%.15f" % r.normalized, "%.1fs" % (time.time() - t0), flush=True)
    return {"workload": name, "n": n, "seed": seed, "n_dofs": sd["n"], "nnz": int(sd["M"].nnz),
            "n_interface_facets": int(sd["n_interface_facets"]), "signals": out}


def main():
    cases = [
        run_case("cfg1"),
        run_case("cfg4", n=16, pick=[0, 1, 2, 3, 13, 58, 119]),
        run_case("cfg3", n=16, pick=[0, 7, 100, 255, 256, 300, 511]),
        run_case("cfg2", n=20),
        run_case("cfg2"),
    ]
    path = os.path.join(os.path.dirname(os.path.abspath(__file__)), "oracle_signals.json")
    with open(path, "w") as fh:
        json.dump({"generator": "tests/golden/make_golden.py", "solver": "oracle.solve_duplicated, SuperLU",
                   "cases": cases}, fh, indent=1)
    print("wrote", path)


if __name__ == "__main__":
    main()
