"""GPU parity for the less common inputs of the solve path, against the CPU
oracle on the same mesh and schedule:

* a non-unit, compartment-discontinuous initial condition (the per-cell field
  of ``DiscontinuousInitialCondition.ipynb`` projected onto P1, handed to
  ``MRI_simulation.solve`` as ``ic``; ``DmriFemLib.py:865-876``), on the FP64
  and the mixed-precision path;
* a whole signal with an anisotropic per-cell diffusion tensor
  (``ImposeDiffusionTensor``, ``DmriFemLib.py:611-616``);
* arbitrary gradient profiles of ``ArbitraryTimeSequence.ipynb:348-449``
  (trapezoid PGSE, sin-OGSE, double PGSE), the oracle building each profile
  from its own piecewise definition;
* one adjoint gradient per parameter kind on the 48^3 layered-sphere mesh
  itself, against central finite differences of the GPU FP64 forward.

Tolerances: FP64 <= 1e-9 relative to the oracle's SuperLU signal, mixed
precision <= 1e-6, adjoint <= 1e-5 relative to the finite difference.
"""

import math

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-9
MIXED_RTOL = 1e-6
ADJ_RTOL = 1e-5


def _ctx(pkg, xyz, tets, reg, nr, D, iT2=None, kp=None):
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, nr)
    ctx.set_coefficients(D, iT2, kp)
    ctx.assemble()
    return ctx


def test_discontinuous_initial_condition(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-8, 8, 10)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.5, -0.5)], [4.5])
    D = np.array([3e-3, 2e-3])
    kp = 5e-5
    # IC_array = [1.0, 0.3]: 1 outside, 0.3 inside, projected onto P1
    u0 = pkg.project_cell_values(pkg.Mesh(xyz, tets), np.where(reg == 1, 0.3, 1.0))
    assert np.ptp(u0) > 0.5
    ctx = _ctx(pkg, xyz, tets, reg, 2, D, None, kp)
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    g = np.array([1.0, 0.0, 0.0])
    bs = (1000.0, 3000.0)
    q = [pkg.sequences.b_to_q(b, p.int4gb()) for b in bs]
    sd = oracle.duplicated_system(xyz, tets, reg, D, 0.0, kp)
    got64 = ctx.solve(q, [g, g], u0=u0, precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
    gotmx = ctx.solve(q, [g, g], u0=u0, precision=pkg.PRECISION_MIXED, rtol=1e-9, max_iterations=20000)
    for k, b in enumerate(bs):
        ref = oracle.solve_duplicated(sd, oracle.PGSE(10600, 43100), q[k], g, 200.0, u0=u0)
        assert abs(got64["S0"] - ref.S0) <= 1e-12 * ref.S0
        n64 = got64["signal"][k] / got64["S0"]
        nmx = gotmx["signal"][k] / gotmx["S0"]
        assert abs(n64 - ref.normalized) <= SIG_RTOL * abs(ref.normalized), (b, n64, ref.normalized)
        assert abs(nmx - ref.normalized) <= MIXED_RTOL * abs(ref.normalized), (b, nmx, ref.normalized)
    # the unit IC gives a different signal (the IC is really used)
    one = ctx.solve(q[:1], [g], precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
    assert abs(one["signal"][0] / one["S0"] - got64["signal"][0] / got64["S0"]) > 1e-4
    ctx.close()


def test_anisotropic_tensor_signal(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 8)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [3.5])
    rng = np.random.default_rng(5)
    L = rng.normal(size=(len(tets), 3, 3)) * 2e-2
    Dt = np.einsum("tij,tkj->tik", L, L) + 1e-3 * np.eye(3)
    D6 = np.stack([Dt[:, 0, 0], Dt[:, 1, 1], Dt[:, 2, 2], Dt[:, 0, 1], Dt[:, 0, 2], Dt[:, 1, 2]], axis=1)
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients([3e-3, 3e-3], None, 3e-5)
    ctx.set_cell_diffusion(D6)
    ctx.assemble()
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    gs = [np.array([1.0, 0.0, 0.0]), np.array([0.0, 0.6, 0.8])]
    q = pkg.sequences.b_to_q(2000.0, p.int4gb())
    sd = oracle.duplicated_system(xyz, tets, reg, Dt, 0.0, 3e-5)
    got64 = ctx.solve([q, q], gs, precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
    gotmx = ctx.solve([q, q], gs, precision=pkg.PRECISION_MIXED, rtol=1e-9, max_iterations=20000)
    refs = [oracle.solve_duplicated(sd, oracle.PGSE(10600, 43100), q, g, 200.0).normalized for g in gs]
    for k in range(2):
        n64 = got64["signal"][k] / got64["S0"]
        nmx = gotmx["signal"][k] / gotmx["S0"]
        assert abs(n64 - refs[k]) <= SIG_RTOL * abs(refs[k]), (k, n64, refs[k])
        assert abs(nmx - refs[k]) <= MIXED_RTOL * abs(refs[k]), (k, nmx, refs[k])
    assert abs(refs[0] - refs[1]) > 1e-3            # the tensor is anisotropic enough to matter
    ctx.close()


def _const(c):
    return lambda s: np.full(np.shape(s), c, dtype=np.float64)


def oracle_trapezoid(d, D):
    """Profile 5 of ArbitraryTimeSequence.ipynb: ramps of delta/3."""
    tau, Dd = d / 3.0, d + D
    return oracle.Sequence([
        (tau, False, lambda s: s / tau), (d - tau, False, _const(1.0)), (d, False, lambda s: -(s - d) / tau),
        (D, False, _const(0.0)), (D + tau, False, lambda s: -(s - D) / tau), (Dd - tau, False, _const(-1.0)),
        (Dd, False, lambda s: (s - Dd) / tau)], Dd, name="trapezoid")


def oracle_sin_ogse(d, D, n=1):
    """Profile 4: sin lobes, the second at tau = (Delta + delta) / 2."""
    om, tau, Dd = 2.0 * math.pi * n / d, (d + D) / 2.0, d + D
    return oracle.Sequence([
        (d, True, lambda s: np.sin(om * s)), (tau, True, _const(0.0)),
        (d + tau, True, lambda s: -np.sin(om * (s - tau)))], Dd, name="sin-OGSE")


def oracle_double_pgse(d, D):
    """Profile 2: two PGSE blocks, the second after a pause of delta."""
    Dd = d + D
    disp = Dd + d
    return oracle.Sequence([
        (d, False, _const(1.0)), (D, False, _const(0.0)), (Dd, False, _const(-1.0)), (disp, False, _const(0.0)),
        (d + disp, False, _const(1.0)), (D + disp, False, _const(0.0)), (Dd + disp, False, _const(-1.0))],
        2 * Dd + d, name="double PGSE")


@pytest.mark.parametrize("name", ["trapezoid", "sin_ogse", "double_pgse"])
def test_arbitrary_profiles(pkg, lib, name):
    d, D = 10600.0, 43100.0
    if name == "trapezoid":
        prof, oseq = pkg.sequences.trapezoid_pgse(d, D), oracle_trapezoid(d, D)
    elif name == "sin_ogse":
        prof, oseq = pkg.sequences.sin_ogse(d, D), oracle_sin_ogse(d, D)
    else:
        d, D = 5000.0, 20000.0
        prof, oseq = pkg.sequences.double_pgse(d, D), oracle_double_pgse(d, D)
    assert abs(prof.T - oseq.T) < 1e-9
    assert abs(prof.int4gb() / oseq.int4gb() - 1.0) < 1e-12
    xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 8)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.5)], [3.0])
    ctx = _ctx(pkg, xyz, tets, reg, 2, [3e-3, 2e-3], None, 2e-5)
    fn, fo = pkg.sequences.profile_samples(prof, 200.0)
    tn, to = oracle.reference_schedule(oseq.T, 200.0)
    assert np.allclose(fn, [oseq.f(t) for t in tn], rtol=0, atol=1e-12)
    assert np.allclose(fo, [oseq.f(t) for t in to], rtol=0, atol=1e-12)
    ctx.set_schedule(fn, fo, 200.0)
    g = np.array([0.48, 0.6, 0.64])
    q = oracle.bvalue_to_q(2500.0, oseq.int4gb())
    sd = oracle.duplicated_system(xyz, tets, reg, np.array([3e-3, 2e-3]), 0.0, 2e-5)
    ref = oracle.solve_duplicated(sd, oseq, q, g, 200.0)
    got64 = ctx.solve([q], [g], precision=pkg.PRECISION_FP64, rtol=1e-13, max_iterations=20000)
    gotmx = ctx.solve([q], [g], precision=pkg.PRECISION_MIXED, rtol=1e-9, max_iterations=20000)
    n64 = got64["signal"][0] / got64["S0"]
    nmx = gotmx["signal"][0] / gotmx["S0"]
    assert abs(n64 - ref.normalized) <= SIG_RTOL * abs(ref.normalized), (name, n64, ref.normalized)
    assert abs(nmx - ref.normalized) <= MIXED_RTOL * abs(ref.normalized), (name, nmx, ref.normalized)
    ctx.close()


def test_adjoint_fd_on_the_48_layered_sphere(pkg, lib):
    """dS/dD, dS/d(1/T2) and dS/dkappa of one signal on the full 48^3 layered
    sphere (129,577 dofs): one parameter per kind against a central difference
    (1e-6 relative step) of the GPU FP64 forward."""
    w = pkg.meshgen.workload("cfg4")
    D = np.asarray(w["D"], np.float64)
    iT2 = np.asarray(w["invT2"], np.float64)
    kp = np.asarray(w["kappa"], np.float64)
    ctx = _ctx(pkg, w["xyz"], w["tets"], w["region"], 4, D, iT2, kp)
    p = w["profiles"][0]
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    b, g, _ = w["signals"][42]
    g = np.asarray(g) / np.linalg.norm(g)
    q = pkg.sequences.b_to_q(b, p.int4gb())
    adj = ctx.adjoint(q, g, rtol=1e-13, max_iterations=20000)

    def sig(Dx, Tx, Kx):
        ctx.set_coefficients(Dx, Tx, Kx)
        ctx.assemble()
        return ctx.solve([q], [g], rtol=1e-13, max_iterations=20000)["signal"][0]

    h = 1e-6
    r = 1
    Dp, Dm = D.copy(), D.copy()
    Dp[r] *= 1 + h
    Dm[r] *= 1 - h
    fd = (sig(Dp, iT2, kp) - sig(Dm, iT2, kp)) / (2 * h * D[r])
    assert abs(adj["dD"][r] - fd) <= ADJ_RTOL * abs(fd), ("D", adj["dD"][r], fd)
    r = 2
    Tp, Tm = iT2.copy(), iT2.copy()
    Tp[r] *= 1 + h
    Tm[r] *= 1 - h
    fd = (sig(D, Tp, kp) - sig(D, Tm, kp)) / (2 * h * iT2[r])
    assert abs(adj["dinvT2"][r] - fd) <= ADJ_RTOL * abs(fd), ("1/T2", adj["dinvT2"][r], fd)
    i, j = 2, 3
    Kp, Km = kp.copy(), kp.copy()
    Kp[i, j] = Kp[j, i] = kp[i, j] * (1 + h)
    Km[i, j] = Km[j, i] = kp[i, j] * (1 - h)
    fd = (sig(D, iT2, Kp) - sig(D, iT2, Km)) / (2 * h * kp[i, j])
    assert abs(adj["dkappa"][i, j] - fd) <= ADJ_RTOL * abs(fd), ("kappa", adj["dkappa"][i, j], fd)
    ctx.close()


def test_device_pointer_solve(pkg, lib):
    """bt_solve_dev with torch CUDA tensors (q, gdir, sequence, u0 in, signals out)
    gives bt_solve's signals bit for bit; host arrays are refused."""
    import torch
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 8)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [3.0])
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients([3e-3, 2e-3], None, 1e-5)
    ctx.assemble()
    seqs = [pkg.sequences.pgse(1000.0, 3000.0), pkg.sequences.cos_ogse(1000.0, 3000.0)]
    fns, fos = zip(*[pkg.sequences.profile_samples(p, 50.0) for p in seqs])
    ctx.set_schedule(np.array(fns), np.array(fos), 50.0)
    q = np.array([pkg.sequences.b_to_q(b, seqs[0].int4gb()) for b in (500.0, 1500.0, 3000.0)])
    g = np.array([[1.0, 0.0, 0.0], [0.0, 0.6, 0.8], [0.48, 0.6, 0.64]])
    sq = np.array([0, 1, 0], np.int32)
    u0 = 1.0 + 0.1 * np.sin(xyz[:, 0])
    for prec in (pkg.PRECISION_FP64, pkg.PRECISION_MIXED):
        ref = ctx.solve(q, g, sq, u0, prec, 1e-12 if prec == pkg.PRECISION_FP64 else 1e-9, 20000, compartments=True)
        out = ctx.solve_dev(torch.tensor(q, device="cuda"), torch.tensor(g, device="cuda"),
                            torch.tensor(sq, device="cuda"), torch.tensor(u0, device="cuda"), prec,
                            1e-12 if prec == pkg.PRECISION_FP64 else 1e-9, 20000, compartments=True)
        assert out["signal"].is_cuda
        assert np.array_equal(out["signal"].cpu().numpy(), ref["signal"])
        assert np.array_equal(out["compartments"].cpu().numpy(), ref["compartments"])
        assert out["S0"] == ref["S0"]
    # host memory is refused
    rc = lib.bt_solve_dev(ctx.h, 1, q.ctypes.data, g.ctypes.data, None, None, 0, 1e-9, 100,
                          torch.zeros(1, dtype=torch.float64, device="cuda").data_ptr(), None, None, None)
    assert rc == 1
    ctx.close()
