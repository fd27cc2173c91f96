"""GPU parity: libbtgpu (through the C ABI) against the CPU oracle.

Tolerances: matrices entrywise <= 1e-13 of the matrix's largest entry (closed
forms, different summation order); FP64 signals <= 1e-9 relative to the
oracle's SuperLU solve (the engine solves each step with COCG to
||r|| <= 1e-12 ||b||).
"""

import math

import numpy as np
import pytest
import scipy.sparse as sps

import oracle

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-9
MAT_RTOL = 1e-13


def make_ctx(pkg, xyz, tets, reg, nr, D, iT2=None, kp=None, rc=None):
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, nr, rc)
    ctx.set_coefficients(D, iT2, kp)
    ctx.assemble()
    return ctx


def layered(pkg, n=6):
    xyz, tets = pkg.meshgen.kuhn_box(-12, 12, n)
    reg = pkg.meshgen.layered_sphere_regions(xyz, tets, [4.0, 7.0, 10.0])
    kp = np.zeros((4, 4))
    for (i, j), v in {(0, 1): 1e-5, (1, 2): 3e-5, (2, 3): 5e-5}.items():
        kp[i, j] = kp[j, i] = v
    D = np.array([1e-3, 2e-3, 3e-3, 3e-3])
    iT2 = 1.0 / np.array([5e4, 8e4, 1e5, np.inf])
    return xyz, tets, reg, D, iT2, kp


def gpu_csr(ctx, values):
    rp, col = ctx.csr()
    n = len(rp) - 1
    return sps.csr_matrix((values, col, rp), shape=(n, n))


@pytest.mark.parametrize("case", ["cylinder", "layers"])
def test_matrices_match_oracle(pkg, lib, case):
    if case == "cylinder":
        xyz, tets = pkg.meshgen.kuhn_box(-10, 10, 7)
        reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.5, -0.3)], [6.0])
        D, iT2, kp = np.array([3e-3, 2e-3]), np.array([0.0, 1e-5]), np.array([[0, 2e-5], [2e-5, 0]])
    else:
        xyz, tets, reg, D, iT2, kp = layered(pkg)
    nr = int(reg.max()) + 1
    ctx = make_ctx(pkg, xyz, tets, reg, nr, D, iT2, kp)
    sd = oracle.duplicated_system(xyz, tets, reg, D, iT2, kp)
    info = ctx.info()
    assert info["n_dofs"] == sd["n"]
    assert info["n_interface_facets"] == sd["n_interface_facets"]
    dv, dc, w = ctx.dofs()
    assert np.array_equal(dv, sd["vertex"]) and np.array_equal(dc, sd["field"])
    assert np.max(np.abs(w - sd["w"])) <= MAT_RTOL * np.abs(sd["w"]).max()
    # sparsity: union of every coupling of the oracle
    P = ((abs(sd["M"]) + abs(sd["R"])) != 0).astype(np.float64)   # cell couplings + interface couplings
    rp, col = ctx.csr()
    G = sps.csr_matrix((np.ones(len(col)), col, rp), shape=P.shape)
    assert G.nnz == P.nnz and G.multiply(P).nnz == P.nnz
    assert all(np.all(np.diff(col[rp[i]:rp[i + 1]]) > 0) for i in range(len(rp) - 1))   # sorted, unique
    for name in ("M", "K", "T", "R", "Jx", "Jy", "Jz"):
        A = gpu_csr(ctx, ctx.matrix(name))
        B = sd[name]
        scale = max(abs(B).max(), 1e-300)
        assert abs(A - B).max() <= MAT_RTOL * scale, name
        assert abs(A - A.T).max() <= MAT_RTOL * scale, name + " symmetric"
    assert math.isclose(info["volume"], sd["volume"], rel_tol=1e-13)
    ctx.close()


def test_anisotropic_cell_tensor(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 5)
    reg = np.zeros(len(tets), np.int32)
    rng = np.random.default_rng(3)
    L = rng.normal(size=(len(tets), 3, 3)) * 1e-2
    Dt = np.einsum("tij,tkj->tik", L, L) + 1e-3 * np.eye(3)
    D6 = np.stack([Dt[:, 0, 0], Dt[:, 1, 1], Dt[:, 2, 2], Dt[:, 0, 1], Dt[:, 0, 2], Dt[:, 1, 2]], axis=1)
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 1)
    ctx.set_coefficients([3e-3])
    ctx.set_cell_diffusion(D6)
    ctx.assemble()
    sd = oracle.duplicated_system(xyz, tets, reg, Dt)
    A = gpu_csr(ctx, ctx.matrix("K"))
    assert abs(A - sd["K"]).max() <= MAT_RTOL * abs(sd["K"]).max()
    ctx.close()


def test_cell_T2_field(pkg, lib):
    """Per-cell 1/T2 (a DG0 T2 field): the T2 mass matrix and a signal against
    the oracle with the same field; the adjoint refuses per-cell T2."""
    xyz, tets, reg, D, iT2, kp = layered(pkg, n=6)
    rng = np.random.default_rng(11)
    iT2c = rng.uniform(0.0, 3e-5, size=len(tets))
    ctx = make_ctx(pkg, xyz, tets, reg, 4, D, iT2, kp)
    ctx.set_cell_T2(iT2c)
    ctx.assemble()
    sd = oracle.duplicated_system(xyz, tets, reg, D, iT2c, kp)
    A = gpu_csr(ctx, ctx.matrix("T"))
    assert abs(A - sd["T"]).max() <= MAT_RTOL * abs(sd["T"]).max()
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    q = pkg.sequences.b_to_q(2000.0, p.int4gb())
    g = np.array([0.6, 0.0, 0.8])
    got = ctx.solve([q], [g], precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
    ref = oracle.solve_duplicated(sd, oracle.PGSE(10600, 43100), q, g, 200.0)
    assert abs(got["signal"][0] / got["S0"] - ref.normalized) <= 1e-9 * abs(ref.normalized)
    with pytest.raises(pkg.BtError):
        ctx.adjoint(q, g)
    ctx.set_cell_T2(None)
    ctx.assemble()
    sd0 = oracle.duplicated_system(xyz, tets, reg, D, iT2, kp)
    assert abs(gpu_csr(ctx, ctx.matrix("T")) - sd0["T"]).max() <= MAT_RTOL * abs(sd0["T"]).max()
    ctx.close()


def test_colouring_is_valid(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 9)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0, 0)], [3.0])
    ctx = make_ctx(pkg, xyz, tets, reg, 2, [3e-3, 3e-3], None, 1e-5)
    col = ctx.colouring()
    assert col.min() >= 0 and ctx.info()["n_colours"] == col.max() + 1
    for c in range(col.max() + 1):
        v = tets[col == c].ravel()
        assert len(np.unique(v)) == len(v), "colour %d has cells sharing a vertex" % c
    ctx.close()


def _profile(pkg, pi, w):
    return w["profiles"][pi]


def test_signals_match_golden(pkg, lib, golden):
    for case in golden["cases"]:
        w = pkg.meshgen.workload(case["workload"], seed=case["seed"], n=case["n"])
        nr = w["n_regions"]
        rc = None if w["multiple"] else np.zeros(nr, np.int32)
        ctx = make_ctx(pkg, w["xyz"], w["tets"], w["region"], nr, w["D"], w["invT2"], w["kappa"], rc)
        info = ctx.info()
        assert info["n_dofs"] == case["n_dofs"]
        fns, fos = zip(*[pkg.sequences.profile_samples(p, w["dt"]) for p in w["profiles"]])
        ctx.set_schedule(np.array(fns), np.array(fos), w["dt"])
        sig = case["signals"]
        q = [s["q"] for s in sig]
        g = [s["gdir"] for s in sig]
        pidx = [s["profile"] for s in sig]
        out = ctx.solve(q, g, pidx, rtol=1e-12, max_iterations=5000, compartments=True)
        for k, s in enumerate(sig):
            got = out["signal"][k] / out["S0"]
            rel = abs(got - s["normalized"]) / abs(s["normalized"])
            assert rel <= SIG_RTOL, (case["workload"], case["n"], s["index"], got, s["normalized"], rel)
            assert np.allclose(out["compartments"][k], s["compartments"], rtol=1e-8, atol=1e-9 * abs(s["signal"]))
        ctx.close()


def test_convergence_test_kat_on_gpu(pkg, lib, kats):
    k = kats["convergence_test_3d_box"]
    s, p = k["setup"], k["printed"]
    xyz, tets = pkg.meshgen.kuhn_box(s["box"][0], s["box"][1], s["cubes_per_axis"])
    mesh = pkg.Mesh(xyz, tets)
    para = pkg.MRI_parameters()
    para.bvalue = s["b"]
    para.delta, para.Delta = s["delta"], s["Delta"]
    para.set_gradient_dir(mesh, *s["gdir"])
    para.T = para.Delta + para.delta
    para.profile = pkg.sequences.pgse(para.delta, para.Delta)
    para.Apply()
    simu = pkg.MRI_simulation()
    simu.k = s["dt"]
    simu.loop = "lt_T"
    dom = pkg.MyDomain(mesh, para)
    dom.Apply()
    dom.D = s["D"]
    lin = pkg.KrylovSolver()
    simu.solve(dom, para, lin)
    assert simu.nsteps == 1100
    norm = simu.signal / simu.voi
    assert "%.6e" % norm == "%.6e" % p["normalized"]
    assert "%.3e" % simu.signal == "%.3e" % p["signal"]
    assert "%.3e" % dom.hmin == "%.3e" % p["hmin"]
    sd = oracle.duplicated_system(xyz, tets, np.zeros(len(tets), np.int32), s["D"])
    ref = oracle.solve_duplicated(sd, oracle.PGSE(s["delta"], s["Delta"]), para.qvalue, s["gdir"], s["dt"],
                                  loop="lt_T")
    assert abs(norm - ref.normalized) <= SIG_RTOL * ref.normalized
    line = pkg.PostProcessing(dom, para, simu, None, logfile=None)
    assert "Normalized signal: 8.440078e-01" in line


def test_b0_and_T2_identities(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 6)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0, 0)], [3.0])
    T2 = 5e4
    ctx = make_ctx(pkg, xyz, tets, reg, 2, [3e-3, 1e-3], [1.0 / T2, 1.0 / T2], 3e-5)
    p = pkg.sequences.pgse(1000, 3000)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    out = ctx.solve([0.0], [1, 0, 0], rtol=1e-13)
    exact = ((1 - 0.5 * 200.0 / T2) / (1 + 0.5 * 200.0 / T2)) ** len(fn)
    assert abs(out["signal"][0] / out["S0"] - exact) < 1e-11
    ctx.set_coefficients([3e-3, 1e-3], None, 3e-5)
    ctx.assemble()
    out = ctx.solve([0.0], [1, 0, 0], rtol=1e-13)
    assert abs(out["signal"][0] / out["S0"] - 1.0) < 1e-12
    ctx.close()


def test_deterministic_bitwise(pkg, lib):
    xyz, tets, reg, D, iT2, kp = layered(pkg, 8)
    runs = []
    for _ in range(2):
        ctx = make_ctx(pkg, xyz, tets, reg, 4, D, iT2, kp)
        p = pkg.sequences.pgse(10600, 43100)
        fn, fo = pkg.sequences.profile_samples(p, 200.0)
        ctx.set_schedule(fn, fo, 200.0)
        q = pkg.sequences.b_to_q(3000.0, p.int4gb())
        out = ctx.solve([q, q], [[1, 0, 0], [0.6, 0.8, 0]], rtol=1e-12)
        runs.append((out["signal"].copy(), ctx.solution(1), ctx.matrix("R")))
        ctx.close()
    assert np.array_equal(runs[0][0], runs[1][0])
    assert np.array_equal(runs[0][1], runs[1][1])
    assert np.array_equal(runs[0][2], runs[1][2])


def test_solution_matches_oracle_field(pkg, lib):
    xyz, tets, reg, D, iT2, kp = layered(pkg, 6)
    ctx = make_ctx(pkg, xyz, tets, reg, 4, D, iT2, kp)
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    q = pkg.sequences.b_to_q(2000.0, p.int4gb())
    ctx.solve([q], [0.0, 0.6, 0.8], rtol=1e-13)
    u = ctx.solution(0)
    sd = oracle.duplicated_system(xyz, tets, reg, D, iT2, kp)
    ref = oracle.solve_duplicated(sd, oracle.PGSE(10600, 43100), q, (0.0, 0.6, 0.8), 200.0)
    assert np.max(np.abs(u - ref.u)) <= 1e-9 * np.max(np.abs(ref.u))
    ctx.close()


def test_errors_are_status_codes(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-2, 2, 3)
    reg = np.zeros(len(tets), np.int32)
    ctx = pkg.Context(0)
    bad = tets.copy()
    bad[0, 0] = len(xyz) + 5
    with pytest.raises(pkg.BtError) as e:
        ctx.mesh_upload(xyz, bad, reg, 1)
    assert e.value.code == 1
    ctx.mesh_upload(xyz, tets, reg, 1)
    with pytest.raises(pkg.BtError) as e:
        ctx.solve([1e-5], [1, 0, 0])
    assert e.value.code == 7                     # BT_ERR_STATE: not assembled
    ctx.set_coefficients([3e-3])
    ctx.assemble()
    p = pkg.sequences.pgse(1000, 3000)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    with pytest.raises(pkg.BtError) as e:
        ctx.solve([pkg.sequences.b_to_q(1000, p.int4gb())], [1, 0, 0], rtol=1e-14, max_iterations=1)
    assert e.value.code == 4                     # BT_ERR_NOT_CONVERGED, kernel left cleanly
    out = ctx.solve([0.0], [1, 0, 0], rtol=1e-12)     # the context is still usable
    assert abs(out["signal"][0] / out["S0"] - 1.0) < 1e-12
    ctx.close()


@pytest.mark.parametrize("case", ["layers", "cylinder"])
def test_crouzeix_raviart_kappa(pkg, lib, case):
    """The per-interface permeability as a Crouzeix-Raviart field (linear on a
    facet whose cell has another interface facet): the interface matrix
    entrywise and an FP64 signal against the oracle's CR mode, and a measurable
    difference from the one-value-per-facet mode on the staircase mesh."""
    if case == "layers":
        xyz, tets, reg, D, iT2, kp = layered(pkg, n=8)
        nr = 4
    else:
        xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 10)
        reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.3, -0.2)], [3.6])
        D, iT2, kp, nr = np.array([3e-3, 2e-3]), np.zeros(2), np.array([[0.0, 4e-5], [4e-5, 0.0]]), 2
    ctx = make_ctx(pkg, xyz, tets, reg, nr, D, iT2, kp)
    ctx.set_kappa_mode("cr")
    ctx.assemble()
    sd = oracle.duplicated_system(xyz, tets, reg, D, iT2, kp, kappa_mode="cr")
    A = gpu_csr(ctx, ctx.matrix("R"))
    assert abs(A - sd["R"]).max() <= MAT_RTOL * abs(sd["R"]).max()
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    q = pkg.sequences.b_to_q(3000.0, p.int4gb())
    g = np.array([0.6, 0.8, 0.0])
    got = ctx.solve([q], [g], precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
    ref = oracle.solve_duplicated(sd, oracle.PGSE(10600, 43100), q, g, 200.0)
    n_cr = got["signal"][0] / got["S0"]
    assert abs(n_cr - ref.normalized) <= SIG_RTOL * abs(ref.normalized), (n_cr, ref.normalized)
    with pytest.raises(pkg.BtError):
        ctx.adjoint(q, g)
    ctx.set_kappa_mode("facet")
    ctx.assemble()
    n_f = ctx.solve([q], [g], precision=pkg.PRECISION_FP64, rtol=1e-13)["signal"][0] / got["S0"]
    assert abs(n_f - n_cr) > 1e-7 * abs(n_cr)
    ctx.close()
