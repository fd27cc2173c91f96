"""GPU: weak pseudo-periodic boundaries (bt_set_periodic) against the CPU oracle
(FP64 path, 1e-9), the mixed path against FP64 (1e-6), the reference-named API,
and the calls that must refuse a periodic context."""

import numpy as np
import pytest

import oracle
import oracle.strong  # noqa: F401

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-9


def periodic_ctx(pkg, xyz, tets, reg, nr, D, kp, pdir, seq, dt):
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, nr)
    ctx.set_coefficients(D, None, kp)
    ctx.assemble()
    ctx.set_periodic(pdir)
    fn, fo = pkg.sequences.profile_samples(seq, dt)
    ctx.set_schedule(fn, fo, dt)
    ctx.set_schedule_phase(pkg.sequences.phase_samples(seq, dt))
    return ctx


def oracle_signal(xyz, tets, reg, D, kp, pdir, q, g, dt, delta, Delta):
    sd = oracle.duplicated_system(xyz, tets, reg, D, 0.0, kp)
    per = oracle.weak_periodic(xyz, tets, np.asarray(reg) % 2, sd["dof"], pdir)
    return oracle.solve_duplicated(sd, oracle.PGSE(delta, Delta), q, g, dt, periodic=per)


@pytest.mark.parametrize("case", ["one", "two"])
def test_fp64_matches_oracle(pkg, lib, case):
    if case == "one":
        xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 8)
        reg = np.zeros(len(tets), np.int32)
        D, kp, nr, pdir = [2e-3], None, 1, [1, 1, 0]
        g = np.array([0.8, 0.6, 0.0])
    else:
        xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 8)
        reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [3.0])
        D, kp, nr, pdir = [3e-3, 1e-3], 3e-5, 2, [1, 0, 1]
        g = np.array([0.3, 0.5, 0.81])
        g /= np.linalg.norm(g)
    delta, Delta, dt = 1000.0, 10000.0, 50.0
    seq = pkg.sequences.pgse(delta, Delta)
    q = pkg.sequences.b_to_q(1000.0, seq.int4gb())
    ctx = periodic_ctx(pkg, xyz, tets, reg, nr, D, kp, pdir, seq, dt)
    info = ctx.periodic_info()
    assert info["active"] == 1 and info["dir"] == pdir and info["n_unmatched"] == 0 and info["n_entries"] > 0
    out = ctx.solve([q], g, rtol=1e-13, max_iterations=20000)
    kpm = None if kp is None else np.array([[0.0, kp], [kp, 0.0]])
    ref = oracle_signal(xyz, tets, reg, D, 0.0 if kpm is None else kpm, pdir, q, g, dt, delta, Delta)
    assert abs(out["signal"][0] - ref.signal) <= SIG_RTOL * abs(ref.signal), (out["signal"][0], ref.signal)
    u = ctx.solution(0)
    assert np.max(np.abs(u - ref.u)) <= 1e-9 * np.max(np.abs(ref.u))
    # the boundary term matters: without it the signal differs by far more
    ctx.set_periodic(None)
    plain = ctx.solve([q], g, rtol=1e-13, max_iterations=20000)["signal"][0]
    assert abs(plain - ref.signal) > 1e-4 * abs(ref.signal)
    ctx.close()


def test_mixed_matches_fp64(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 10)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [3.0])
    seq = pkg.sequences.pgse(1000.0, 10000.0)
    ctx = periodic_ctx(pkg, xyz, tets, reg, 2, [3e-3, 1e-3], 3e-5, [1, 0, 0], seq, 50.0)
    q = np.array([pkg.sequences.b_to_q(b, seq.int4gb()) for b in (500.0, 1000.0, 2000.0, 3000.0)])
    g = np.array([[1.0, 0.0, 0.0], [0.6, 0.8, 0.0], [0.0, 0.6, 0.8], [1.0, 0.0, 0.0]])
    ref = ctx.solve(q, g, rtol=1e-13, max_iterations=20000)["signal"]
    mix = ctx.solve(q, g, precision=pkg.PRECISION_MIXED, rtol=1e-9, max_iterations=20000)["signal"]
    assert np.max(np.abs(mix - ref) / np.abs(ref)) <= 1e-6, np.abs(mix - ref) / np.abs(ref)
    ctx.close()


def test_switching_off_restores_the_plain_solve(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 6)
    reg = np.zeros(len(tets), np.int32)
    seq = pkg.sequences.pgse(1000.0, 10000.0)
    q = pkg.sequences.b_to_q(1000.0, seq.int4gb())
    ctx = periodic_ctx(pkg, xyz, tets, reg, 1, [2e-3], None, [0, 0, 1], seq, 50.0)
    a = ctx.solve([q], [0, 0, 1], rtol=1e-13)["signal"][0]
    ctx.set_periodic([0, 0, 0])
    b = ctx.solve([q], [0, 0, 1], rtol=1e-13)["signal"][0]
    fresh = pkg.Context(0)
    fresh.mesh_upload(xyz, tets, reg, 1)
    fresh.set_coefficients([2e-3])
    fresh.assemble()
    fn, fo = pkg.sequences.profile_samples(seq, 50.0)
    fresh.set_schedule(fn, fo, 50.0)
    c = fresh.solve([q], [0, 0, 1], rtol=1e-13)["signal"][0]
    assert b == c and a != b
    assert ctx.periodic_info()["active"] == 0
    fresh.close()
    ctx.close()


def test_refusals(pkg, lib):
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 4)
    reg = np.zeros(len(tets), np.int32)
    seq = pkg.sequences.pgse(1000.0, 10000.0)
    q = pkg.sequences.b_to_q(1000.0, seq.int4gb())
    ctx = periodic_ctx(pkg, xyz, tets, reg, 1, [2e-3], None, [1, 0, 0], seq, 50.0)
    with pytest.raises(pkg.BtError) as e:
        ctx.adjoint(q, [1, 0, 0])
    assert e.value.code == 7
    fn, fo = pkg.sequences.profile_samples(seq, 50.0)
    ctx.set_schedule(fn, fo, 50.0)             # clears the phase schedule
    with pytest.raises(pkg.BtError) as e:
        ctx.solve([q], [1, 0, 0])
    assert e.value.code == 7
    with pytest.raises(pkg.BtError) as e:
        ctx.set_periodic([2, 0, 0])
    assert e.value.code == 1
    ctx.close()


def test_reference_api(pkg, lib):
    """MyDomain.PeriodicDir through MRI_simulation.solve, against the oracle."""
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 6)
    mesh = pkg.Mesh(xyz, tets)
    para = pkg.MRI_parameters()
    para.bvalue, para.delta, para.Delta = 1000, 1000, 10000
    para.set_gradient_dir(mesh, 1, 0, 0)
    para.Apply()
    dom = pkg.MyDomain(mesh, para)
    dom.PeriodicDir = [1, 0, 0]
    dom.D = 2e-3
    dom.Apply()
    sim = pkg.MRI_simulation()
    sim.k = 50
    sim.solve(dom, para)
    reg = np.zeros(len(tets), np.int32)
    ref = oracle_signal(xyz, tets, reg, [2e-3], 0.0, [1, 0, 0], para.qvalue, [1, 0, 0], 50.0, 1000.0, 10000.0)
    assert abs(sim.signal - ref.signal) <= SIG_RTOL * abs(ref.signal)
    # IsDomainPeriodic = True: the strong form (uniform solution of the homogeneous box)
    dom.IsDomainPeriodic = True
    dom.Apply()
    sim.solve(dom, para)
    exact = oracle.strong.uniform_box_signal(1000.0, 2e-3, 0.0, oracle.PGSE(1000.0, 10000.0), para.qvalue, 50.0)
    assert abs(sim.signal - exact) <= SIG_RTOL * abs(exact)
