"""Golden fixtures on meshes shipped with the reference.

Run from the repository root, giving the reference checkout's root as the
argument or in the environment variable DMRI_REFERENCE:
    python tests/golden/make_reference_mesh_fixtures.py <reference root>
Reads comri/meshes/cyl6_r_3E_6_vol.msh.zip and cyl12_r_3E_6_vol.msh.zip of the
reference with meshfiles.read_msh (the gmsh 2.2 files the reference's
GCloud/Preprocessing scripts use; single compartment: every physical tag is 0),
stores their vertices and tetrahedra in reference_meshes.npz and the FP64 oracle
signals (SuperLU per distinct step matrix) in reference_mesh_signals.json.
Workload: D = 3e-3 um^2/us, no T2 decay, PGSE delta = 10600 us, Delta = 43100
us, dt = 200 us (270 steps), b in {1000, 3000} s/mm^2 along x and along the
cylinder axis z.
"""

import importlib
import json
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)
import oracle  # noqa: E402

pkg = importlib.import_module("dmri-fem-cloud_gb300")
NAMES = ["cyl6_r_3E_6_vol", "cyl12_r_3E_6_vol"]


def main(ref_root):
    REF = os.path.join(ref_root, "comri", "meshes")
    arrays, cases = {}, []
    prof = oracle.PGSE(10600, 43100)
    for name in NAMES:
        d = pkg.meshfiles.read_msh(os.path.join(REF, name + ".msh.zip"))
        xyz, tets = d["xyz"], d["tets"]
        arrays[name + "_xyz"] = xyz
        arrays[name + "_tets"] = tets
        region = np.zeros(len(tets), np.int32)
        sd = oracle.duplicated_system(xyz, tets, region, np.array([3e-3]), 0.0, 0.0, field=np.zeros(len(tets), np.int64))
        sig = []
        for b in (1000.0, 3000.0):
            for g in ((1.0, 0.0, 0.0), (0.0, 0.0, 1.0)):
                q = oracle.bvalue_to_q(b, prof.int4gb())
                r = oracle.solve_duplicated(sd, prof, q, np.array(g), 200.0)
                sig.append({"b": b, "q": q, "gdir": list(g), "signal": r.signal, "S0": r.S0,
                            "normalized": r.signal / r.S0})
                print(name, b, g, r.signal / r.S0, flush=True)
        cases.append({"mesh": name, "n_vertices": len(xyz), "n_cells": len(tets), "signals": sig})
    np.savez_compressed(os.path.join(ROOT, "tests", "golden", "reference_meshes.npz"), **arrays)
    with open(os.path.join(ROOT, "tests", "golden", "reference_mesh_signals.json"), "w") as fh:
        json.dump({"workload": "D=3e-3, PGSE 10600/43100 us, dt=200 us, 270 steps", "cases": cases}, fh, indent=1)


if __name__ == "__main__":
    root = sys.argv[1] if len(sys.argv) > 1 else os.environ.get("DMRI_REFERENCE")
    if not root or not os.path.isdir(root):
        sys.exit("give the reference checkout's root as the argument or in DMRI_REFERENCE")
    main(root)
