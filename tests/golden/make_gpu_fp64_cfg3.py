"""FP64 reference signals of every signal of the eight-cylinder 64^3 workload.

Run on a GPU from the repository root:  python tests/golden/make_gpu_fp64_cfg3.py [out.json]
Writes tests/golden/gpu_fp64_cfg3_signals.json (or out.json): the normalised signal of all
512 signals (64 Fibonacci directions x 8 b-values, PGSE and cos-OGSE) from the
plain FP64 path (libbtgpu's FP64 COCG stepper, ||r|| <= 1e-12 ||b|| every step).
The CPU oracle cannot integrate this 311,499-dof workload in reasonable time
(SuperLU per step); the FP64 path itself is pinned to the oracle at 1e-9 on the
full 40^3 workload and on a 16^3 version of this one (tests/test_gpu_parity.py).
bench.py's ``batched`` leg states the mixed path's error against these values
for every signal, and re-runs a spread sample of them live.
"""

import importlib
import json
import os
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)


def main():
    pkg = importlib.import_module("dmri-fem-cloud_gb300")
    pkg._native.load(pkg.build())
    w = pkg.meshgen.workload("cfg3")
    prof = w["profiles"]
    fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in prof])
    int4 = [p.int4gb() for p in prof]
    sig = w["signals"]
    q = np.array([pkg.sequences.b_to_q(b, int4[pi]) for b, _, pi in sig])
    g = np.array([gd for _, gd, _ in sig], np.float64)
    g /= np.linalg.norm(g, axis=1, keepdims=True)
    pidx = np.array([pi for _, _, pi in sig], np.int32)
    ctx = pkg.Context(0)
    ctx.mesh_upload(w["xyz"], w["tets"], w["region"], w["n_regions"], None)
    ctx.set_coefficients(w["D"], w["invT2"], w["kappa"])
    ctx.assemble()
    ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])
    t0 = time.time()
    out = ctx.solve(q, g, pidx, None, pkg.PRECISION_FP64, 1e-12, 20000)
    info = ctx.info()
    ctx.close()
    res = {"generator": "tests/golden/make_gpu_fp64_cfg3.py", "workload": "cfg3", "seed": 0,
           "solver": "libbtgpu FP64 path, COCG rtol 1e-12 per step", "n_dofs": info["n_dofs"], "nnz": info["nnz"],
           "b": [s[0] for s in sig], "profile": pidx.tolist(), "S0": out["S0"],
           "signal": out["signal"].tolist(), "normalized": (out["signal"] / out["S0"]).tolist(),
           "iterations": out["stats"]["total_iterations"], "seconds": time.time() - t0}
    path = sys.argv[1] if len(sys.argv) > 1 else os.path.join(os.path.dirname(os.path.abspath(__file__)),
                                                               "gpu_fp64_cfg3_signals.json")
    with open(path, "w") as fh:
        json.dump(res, fh, indent=0)
    print("wrote", path, "in %.0f s" % res["seconds"])


if __name__ == "__main__":
    main()
