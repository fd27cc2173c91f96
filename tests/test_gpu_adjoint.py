"""GPU: discrete-adjoint gradients of the FP64 solve (bt_adjoint) against
central finite differences with a 1e-6 relative step, of the GPU forward and of
the CPU oracle (tolerance 1e-5 relative to the gradient's scale), and against
the FP64 tangent-linear run (bt_tangent, 1e-8)."""

import numpy as np
import pytest

import oracle

pytestmark = pytest.mark.gpu

ADJ_RTOL = 1e-5


def layered_case(pkg, n=8):
    xyz, tets = pkg.meshgen.kuhn_box(-12, 12, n)
    reg = pkg.meshgen.layered_sphere_regions(xyz, tets, [4.0, 7.0, 10.0])
    D = np.array([1e-3, 2e-3, 3e-3, 3e-3])
    invT2 = 1.0 / np.array([5e4, 8e4, 1e5, np.inf])
    kp = np.zeros((4, 4))
    for (i, j), v in {(0, 1): 1e-5, (1, 2): 3e-5, (2, 3): 5e-5}.items():
        kp[i, j] = kp[j, i] = v
    return xyz, tets, reg, D, invT2, kp


def make(pkg, xyz, tets, reg, D, invT2, kp):
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 4)
    ctx.set_coefficients(D, invT2, kp)
    ctx.assemble()
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    return ctx, pkg.sequences.b_to_q(3000.0, p.int4gb())


G = np.array([0.3, 0.8, 0.52])
G = G / np.linalg.norm(G)


def signal(ctx, q, D, invT2, kp):
    ctx.set_coefficients(D, invT2, kp)
    ctx.assemble()
    return ctx.solve([q], G, rtol=1e-14, max_iterations=20000)["signal"][0]


def test_adjoint_matches_finite_differences(pkg, lib):
    xyz, tets, reg, D, invT2, kp = layered_case(pkg)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    adj = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000)
    base = signal(ctx, q, D, invT2, kp)
    assert abs(adj["signal"] - base) <= 1e-10 * abs(base)
    h = 1e-6
    scale = {"D": np.max(np.abs(adj["dD"] * D)), "T": np.max(np.abs(adj["dinvT2"] * invT2)),
             "K": max(abs(adj["dkappa"][i, j] * kp[i, j]) for i, j in ((0, 1), (1, 2), (2, 3)))}
    for r in range(4):
        Dp, Dm = D.copy(), D.copy()
        Dp[r] *= 1 + h
        Dm[r] *= 1 - h
        fd = (signal(ctx, q, Dp, invT2, kp) - signal(ctx, q, Dm, invT2, kp)) / (2 * h * D[r])
        assert abs(adj["dD"][r] - fd) * D[r] <= ADJ_RTOL * scale["D"], ("D", r, adj["dD"][r], fd)
    for r in range(3):                       # region 3 has no T2 decay (1/T2 = 0)
        Tp, Tm = invT2.copy(), invT2.copy()
        Tp[r] *= 1 + h
        Tm[r] *= 1 - h
        fd = (signal(ctx, q, D, Tp, kp) - signal(ctx, q, D, Tm, kp)) / (2 * h * invT2[r])
        assert abs(adj["dinvT2"][r] - fd) * invT2[r] <= ADJ_RTOL * scale["T"], ("T2", r, adj["dinvT2"][r], fd)
    for i, j in ((0, 1), (1, 2), (2, 3)):
        Kp, Km = kp.copy(), kp.copy()
        Kp[i, j] = Kp[j, i] = kp[i, j] * (1 + h)
        Km[i, j] = Km[j, i] = kp[i, j] * (1 - h)
        fd = (signal(ctx, q, D, invT2, Kp) - signal(ctx, q, D, invT2, Km)) / (2 * h * kp[i, j])
        assert abs(adj["dkappa"][i, j] - fd) * kp[i, j] <= ADJ_RTOL * scale["K"], ("kappa", i, j)
        assert adj["dkappa"][i, j] == adj["dkappa"][j, i]
    assert np.all(adj["dkappa"][[0, 0, 1], [2, 3, 3]] == 0.0)     # no interface between these regions
    ctx.close()


def test_adjoint_matches_oracle_fd(pkg, lib):
    """One gradient against the CPU oracle's central difference (SuperLU)."""
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=6)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    adj = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000)
    h = 1e-6
    vals = []
    for sgn in (1, -1):
        Kx = kp.copy()
        Kx[1, 2] = Kx[2, 1] = kp[1, 2] * (1 + sgn * h)
        sd = oracle.duplicated_system(xyz, tets, reg, D, invT2, Kx)
        vals.append(oracle.solve_duplicated(sd, oracle.PGSE(10600, 43100), q, G, 200.0).signal)
    fd = (vals[0] - vals[1]) / (2 * h * kp[1, 2])
    assert abs(adj["dkappa"][1, 2] - fd) <= ADJ_RTOL * abs(fd)
    ctx.close()


def test_checkpoint_stride_invariance_and_autograd(pkg, lib):
    import torch
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=6)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    a = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000, stride=1)
    b = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000, stride=0)
    c = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000, stride=270)
    for k in ("dD", "dinvT2", "dkappa"):
        ref = np.max(np.abs(a[k]))
        assert np.max(np.abs(a[k] - b[k])) <= 1e-9 * ref and np.max(np.abs(a[k] - c[k])) <= 1e-9 * ref
    from importlib import import_module
    ag = import_module(pkg.__name__ + ".autograd")
    Dt = torch.tensor(D, requires_grad=True)
    Tt = torch.tensor(invT2, requires_grad=True)
    Kt = torch.tensor(kp, requires_grad=True)
    s = ag.BlochTorreySignal.apply(Dt, Tt, Kt, ctx, q, G, 0)
    s.backward()
    S0 = ctx.info()["volume"]
    assert abs(float(s.detach()) - a["signal"] / S0) <= 1e-12
    assert np.allclose(Dt.grad.numpy(), a["dD"] / S0, rtol=1e-9, atol=0)
    assert np.allclose(Kt.grad.numpy(), a["dkappa"] / S0, rtol=1e-9, atol=0)
    ctx.close()


def test_tangent_linear_matches_adjoint(pkg, lib):
    """The FP64 tangent-linear run (forward mode, one parameter at a time) and the
    discrete adjoint give the same derivatives: both are exact derivatives of the
    discrete solve, so they agree to solver precision (1e-8 relative)."""
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=6)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    adj = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000)
    checks = [("D", r, 0, adj["dD"][r]) for r in range(4)]
    checks += [("invT2", r, 0, adj["dinvT2"][r]) for r in range(4)]
    checks += [("kappa", i, j, adj["dkappa"][i, j]) for i, j in ((0, 1), (1, 2), (2, 3))]
    scale = {"D": np.max(np.abs(adj["dD"])), "invT2": np.max(np.abs(adj["dinvT2"])),
             "kappa": np.max(np.abs(adj["dkappa"]))}
    for name, i, j, ref in checks:
        t = ctx.tangent(q, G, name, i, j, rtol=1e-14, max_iterations=20000)
        assert abs(t["signal"] - adj["signal"]) <= 1e-12 * abs(adj["signal"])
        assert abs(t["d"] - ref) <= 1e-8 * scale[name], (name, i, j, t["d"], ref)
    # assembled matrices are untouched by the indicator assembly
    again = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000)
    assert again["signal"] == adj["signal"]
    ctx.close()


def test_batched_mixed_adjoint_matches_fp64(pkg, lib):
    """bt_adjoint_batch (mixed precision, several signals in one set of launches,
    the backward sweep run by the batched stepper) against the FP64 adjoint of
    each signal: gradients within 1e-5 of their scale, signals within 1e-6."""
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=6)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    qs = np.array([q, 0.7 * q, 1.2 * q])
    gs = np.array([G, [1.0, 0.0, 0.0], [0.0, 0.6, 0.8]])
    refs = [ctx.adjoint(qs[i], gs[i], rtol=1e-14, max_iterations=20000) for i in range(3)]
    for stride in (0, 7):
        out = ctx.adjoint_batch(qs, gs, rtol=1e-9, stride=stride)
        for i, ref in enumerate(refs):
            assert abs(out["signal"][i] - ref["signal"]) <= 1e-6 * abs(ref["signal"])
            for k in ("dD", "dinvT2", "dkappa"):
                scale = np.max(np.abs(ref[k]))
                err = np.max(np.abs(out[k][i] - ref[k]))
                assert err <= 1e-5 * scale, (stride, i, k, err / scale)
    ctx.close()


def test_batched_autograd_and_16_cubed_layers(pkg, lib):
    """The batched adjoint on a 16^3 layered sphere (a finer mesh than the other
    adjoint tests) against the FP64 adjoint of a spread of its signals, and the
    batched torch.autograd.Function: its backward equals the contraction of the
    incoming gradient with the per-signal FP64 derivatives, and gradients come
    back on the parameters' device and dtype."""
    import torch
    from importlib import import_module
    ag = import_module(pkg.__name__ + ".autograd")
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=16)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    dirs = pkg.meshgen.fibonacci_directions(6)
    qs = np.array([q * f for f in (0.6, 0.8, 1.0, 1.0, 1.2, 0.9)])
    refs = [ctx.adjoint(qs[i], dirs[i], rtol=1e-13, max_iterations=20000) for i in range(6)]
    dev = torch.device("cuda", 0)
    Dt = torch.tensor(D, dtype=torch.float32, device=dev, requires_grad=True)
    Tt = torch.tensor(invT2, dtype=torch.float64, requires_grad=True)
    Kt = torch.tensor(kp, dtype=torch.float64, device=dev, requires_grad=True)
    s = ag.BlochTorreySignals.apply(Dt, Tt, Kt, ctx, qs, dirs, None)
    assert s.shape == (6,) and s.device == dev and s.dtype == torch.float32
    wts = torch.linspace(0.5, 1.5, 6, dtype=torch.float32, device=dev)
    (s * wts).sum().backward()
    assert Dt.grad.device == dev and Dt.grad.dtype == torch.float32 and Tt.grad.device.type == "cpu"
    S0 = ctx.info()["volume"]
    w = wts.cpu().double().numpy()
    for key, got in (("dD", Dt.grad), ("dinvT2", Tt.grad), ("dkappa", Kt.grad)):
        ref = sum(w[i] * refs[i][key] for i in range(6)) / S0
        scale = max(np.max(np.abs(refs[i][key])) for i in range(6)) / S0
        assert np.max(np.abs(got.detach().cpu().double().numpy() - ref)) <= 1e-5 * scale * w.sum(), key
    for i in range(6):
        assert abs(float(s[i]) - refs[i]["signal"] / S0) <= 1e-6 * abs(refs[i]["signal"] / S0) + 1e-7
    ctx.close()


def test_multi_mesh_adjoint_matches_fp64(pkg, lib):
    """bt_adjoint_multi on a scaled-down uneven batch (seeded cylinder boxes of
    6^3 ... 12^3 cubes sharing launches, plus one 28^3 box that runs alone):
    every signal's gradients within 1e-5 of their scale of the FP64 adjoint of
    that signal on its own mesh, signals within 1e-6."""
    meshes = pkg.meshgen.uneven_meshes(count=4, seed=3, nmin=6, nmax=12, cube=1.5)
    meshes.append(pkg.meshgen.uneven_meshes(count=1, seed=4, nmin=28, nmax=28, cube=1.0)[0])
    p = pkg.sequences.pgse(10600, 43100)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctxs, qs, gs = [], [], []
    dirs = pkg.meshgen.fibonacci_directions(3)
    for m in meshes:
        c = pkg.Context(0)
        c.mesh_upload(m["xyz"], m["tets"], m["region"], 2)
        c.set_coefficients(m["D"], None, m["kappa"])
        c.assemble()
        c.set_schedule(fn, fo, 200.0)
        ctxs.append(c)
        qs.append([pkg.sequences.b_to_q(b, p.int4gb()) for b in (1000.0, 2500.0, 4000.0)])
        gs.append(dirs)
    out = pkg.adjoint_multi(ctxs, qs, gs, rtol=1e-9)
    for k, c in enumerate(ctxs):
        for i in range(3):
            ref = c.adjoint(qs[k][i], gs[k][i], rtol=1e-13, max_iterations=20000)
            assert abs(out["signal"][k][i] - ref["signal"]) <= 1e-6 * abs(ref["signal"]), (k, i)
            for key in ("dD", "dinvT2", "dkappa"):
                scale = np.max(np.abs(ref[key]))
                if scale == 0.0:
                    assert np.all(out[key][k][i] == 0.0), (k, i, key)
                    continue
                err = np.max(np.abs(out[key][k][i] - ref[key]))
                assert err <= 1e-5 * scale, (k, i, key, err / scale)
    for c in ctxs:
        c.close()


def test_cell_field_gradients(pkg, lib):
    """bt_adjoint_cells: the per-cell derivatives sum to the per-region ones
    (isotropic D: xx + yy + zz of the region's cells; 1/T2), and with a per-cell
    anisotropic tensor and per-cell T2 they match central differences of the
    GPU forward (one component or 1/T2 moved on all cells of a region); the
    autograd form returns them."""
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=6)
    ctx, q = make(pkg, xyz, tets, reg, D, invT2, kp)
    adj = ctx.adjoint(q, G, rtol=1e-14, max_iterations=20000)
    cel = ctx.adjoint_cells(q, G, rtol=1e-14, max_iterations=20000)
    assert abs(cel["signal"] - adj["signal"]) <= 1e-12 * abs(adj["signal"])
    iso = cel["dD_cell"][:, :3].sum(axis=1)
    for r in range(4):
        m = reg == r
        assert abs(iso[m].sum() - adj["dD"][r]) <= 1e-10 * np.max(np.abs(adj["dD"]))
        assert abs(cel["dinvT2_cell"][m].sum() - adj["dinvT2"][r]) <= 1e-10 * np.max(np.abs(adj["dinvT2"]))
    assert np.allclose(cel["dkappa"], adj["dkappa"], rtol=1e-12, atol=1e-12 * np.max(np.abs(adj["dkappa"])))
    # anisotropic per-cell field
    rng = np.random.default_rng(3)
    n_t = len(tets)
    D6 = np.zeros((n_t, 6))
    D6[:, :3] = D[reg][:, None] * (1.0 + 0.3 * rng.random((n_t, 3)))
    D6[:, 3:] = D[reg][:, None] * 0.1 * (rng.random((n_t, 3)) - 0.5)
    iT = invT2[reg] + 1e-5 * rng.random(n_t)
    ctx.set_cell_diffusion(D6)
    ctx.set_cell_T2(iT)
    ctx.assemble()
    cel = ctx.adjoint_cells(q, G, rtol=1e-14, max_iterations=20000)

    def sig6(D6x, iTx):
        ctx.set_cell_diffusion(D6x)
        ctx.set_cell_T2(iTx)
        ctx.assemble()
        return ctx.solve([q], G, rtol=1e-14, max_iterations=20000)["signal"][0]

    # central differences of a component over the cells of one region (a single
    # cell's derivative is below the differences' rounding)
    base = sig6(D6, iT)
    assert abs(base - cel["signal"]) <= 1e-10 * abs(base)
    for r, k in ((1, 0), (1, 3), (2, 5), (0, 4)):
        m = reg == r
        h = 1e-6 * 3e-3
        Dp, Dm = D6.copy(), D6.copy()
        Dp[m, k] += h
        Dm[m, k] -= h
        fd = (sig6(Dp, iT) - sig6(Dm, iT)) / (2 * h)
        ad = cel["dD_cell"][m, k].sum()
        scale = np.max(np.abs([cel["dD_cell"][reg == rr, kk].sum() for rr in range(4) for kk in range(6)]))
        assert abs(ad - fd) <= ADJ_RTOL * scale, (r, k, ad, fd)
    for r in (1, 2):
        m = reg == r
        h = 1e-6 * 1e-5
        Tp, Tm = iT.copy(), iT.copy()
        Tp[m] += h
        Tm[m] -= h
        fd = (sig6(D6, Tp) - sig6(D6, Tm)) / (2 * h)
        ad = cel["dinvT2_cell"][m].sum()
        scale = np.max(np.abs([cel["dinvT2_cell"][reg == rr].sum() for rr in range(4)]))
        assert abs(ad - fd) <= ADJ_RTOL * scale, (r, ad, fd)
    # autograd over the fields
    import importlib
    import torch
    ag = importlib.import_module(pkg.__name__ + ".autograd")
    Dt = torch.tensor(D6, requires_grad=True)
    Tt = torch.tensor(iT, requires_grad=True)
    s = ag.BlochTorreyCellField.apply(Dt, Tt, ctx, q, G, 0)
    s.backward()
    S0 = ctx.info()["volume"]
    # (the autograd form runs the adjoint at its default rtol 1e-13, the reference above at 1e-14)
    gs = np.max(np.abs(cel["dD_cell"])) / S0
    assert np.max(np.abs(Dt.grad.numpy() - cel["dD_cell"] / S0)) <= 1e-8 * gs
    gt = np.max(np.abs(cel["dinvT2_cell"])) / S0
    assert np.max(np.abs(Tt.grad.numpy() - cel["dinvT2_cell"] / S0)) <= 1e-8 * gt
    ctx.close()


def test_batched_cell_field_vjp(pkg, lib):
    """bt_adjoint_batch_cells: the per-cell gradients of sum_s w_s S_s from the
    batched mixed adjoint against the weighted sum of the FP64 per-cell adjoints
    (1e-5 of the gradient scale), with a per-cell anisotropic tensor and T2; the
    autograd form over the fields returns them."""
    xyz, tets, reg, D, invT2, kp = layered_case(pkg, n=6)
    ctx, q0 = make(pkg, xyz, tets, reg, D, invT2, kp)
    rng = np.random.default_rng(5)
    n_t = len(tets)
    D6 = np.zeros((n_t, 6))
    D6[:, :3] = D[reg][:, None] * (1.0 + 0.3 * rng.random((n_t, 3)))
    D6[:, 3:] = D[reg][:, None] * 0.1 * (rng.random((n_t, 3)) - 0.5)
    iT = invT2[reg] + 1e-5 * rng.random(n_t)
    ctx.set_cell_diffusion(D6)
    ctx.set_cell_T2(iT)
    ctx.assemble()
    p = pkg.sequences.pgse(10600, 43100)
    qs = np.array([pkg.sequences.b_to_q(b, p.int4gb()) for b in (1000.0, 2000.0, 3000.0)])
    gs = np.array([[1.0, 0.0, 0.0], [0.0, 0.6, 0.8], G])
    w = np.array([0.7, -1.3, 2.1])
    bat = ctx.adjoint_batch_cells(qs, gs, w, rtol=1e-9)
    ref6 = np.zeros((n_t, 6))
    refT = np.zeros(n_t)
    refK = np.zeros((4, 4))
    for i in range(3):
        c = ctx.adjoint_cells(qs[i], gs[i], rtol=1e-13, max_iterations=20000)
        assert abs(bat["signal"][i] - c["signal"]) <= 1e-6 * abs(c["signal"])
        ref6 += w[i] * c["dD_cell"]
        refT += w[i] * c["dinvT2_cell"]
        refK += w[i] * c["dkappa"]
    assert np.max(np.abs(bat["dD_cell"] - ref6)) <= ADJ_RTOL * np.max(np.abs(ref6))
    assert np.max(np.abs(bat["dinvT2_cell"] - refT)) <= ADJ_RTOL * np.max(np.abs(refT))
    assert np.max(np.abs(bat["dkappa"] - refK)) <= ADJ_RTOL * np.max(np.abs(refK))
    import importlib
    import torch
    ag = importlib.import_module(pkg.__name__ + ".autograd")
    Dt = torch.tensor(D6, requires_grad=True)
    Tt = torch.tensor(iT, requires_grad=True)
    s = ag.BlochTorreyCellFields.apply(Dt, Tt, ctx, qs, gs, None)
    (s * torch.tensor(w)).sum().backward()
    S0 = ctx.info()["volume"]
    assert np.max(np.abs(Dt.grad.numpy() - ref6 / S0)) <= ADJ_RTOL * np.max(np.abs(ref6)) / S0
    assert np.max(np.abs(Tt.grad.numpy() - refT / S0)) <= ADJ_RTOL * np.max(np.abs(refT)) / S0
    ctx.close()
