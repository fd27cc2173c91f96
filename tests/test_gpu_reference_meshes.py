"""GPU: meshes shipped with the reference (gmsh files read by meshfiles, stored
as fixtures by tests/golden/make_reference_mesh_fixtures.py) against the FP64
oracle: FP64 path <= 1e-9, mixed path <= 1e-6 relative signal error."""

import json
import os

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def test_reference_meshes_match_oracle(pkg, lib):
    arrays = np.load(os.path.join(GOLDEN, "reference_meshes.npz"))
    cases = json.load(open(os.path.join(GOLDEN, "reference_mesh_signals.json")))["cases"]
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    for case in cases:
        xyz, tets = arrays[case["mesh"] + "_xyz"], arrays[case["mesh"] + "_tets"]
        ctx = pkg.Context(0)
        ctx.mesh_upload(xyz, tets, np.zeros(len(tets), np.int32), 1, np.zeros(1, np.int32))
        ctx.set_coefficients([3e-3])
        ctx.assemble()
        ctx.set_schedule(fn, fo, 200.0)
        q = [s["q"] for s in case["signals"]]
        g = [s["gdir"] for s in case["signals"]]
        ref = np.array([s["normalized"] for s in case["signals"]])
        o64 = ctx.solve(q, g, precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
        omx = ctx.solve(q, g, precision=pkg.PRECISION_MIXED, rtol=1e-9)
        assert np.max(np.abs(o64["signal"] / o64["S0"] - ref) / np.abs(ref)) <= 1e-9, case["mesh"]
        assert np.max(np.abs(omx["signal"] / omx["S0"] - ref) / np.abs(ref)) <= 1e-6, case["mesh"]
        ctx.close()


def test_mesh_file_round_trip_solves_identically(pkg, lib, tmp_path):
    """A mesh written to a gmsh file and read back gives bitwise the same signals."""
    w = pkg.meshgen.workload("cfg2", n=10)
    path = tmp_path / "cfg2.msh"
    pkg.meshfiles.write_msh2(path, w["xyz"], w["tets"], w["region"])
    m = pkg.Mesh.read(path)
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    q = pkg.sequences.b_to_q(3000.0, p.int4gb())
    out = []
    for xyz, tets, reg in ((w["xyz"], w["tets"], w["region"]), (m.xyz, m.tets, m.markers)):
        ctx = pkg.Context(0)
        ctx.mesh_upload(xyz, tets, reg, 2)
        ctx.set_coefficients(w["D"], None, w["kappa"])
        ctx.assemble()
        ctx.set_schedule(fn, fo, 200.0)
        out.append(ctx.solve([q], [[0.0, 1.0, 0.0]], precision=pkg.PRECISION_FP64, rtol=1e-12)["signal"])
        ctx.close()
    assert np.array_equal(out[0], out[1])
