"""GPU: failure detection without a GPU fault.

* Every device-side wait of the persistent steppers is bounded.  The option
  ``test.stall_first_wait`` makes a solve's first wait spin on a word that
  nothing writes, so it runs out after ``wait.limit_ns``: the call must return
  BT_ERR_TIMEOUT, and after the options are restored the same context must
  solve normally (bitwise the same signal as before).
* Invalid inputs (NaN or negative coefficients, bad schedules, non-finite
  gradients) are rejected on the host with BT_ERR_INVALID before any work is
  queued, and leave the context usable.
* An iteration cap that cannot be met ends the solve with BT_ERR_NOT_CONVERGED
  on the FP64 and on the mixed-precision path.
"""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

BT_ERR_INVALID, BT_ERR_NOT_CONVERGED, BT_ERR_TIMEOUT = 1, 4, 6


def _setup(pkg):
    xyz, tets = pkg.meshgen.kuhn_box(-5, 5, 6)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.0, 0.0)], [2.5])
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients([3e-3, 2e-3], None, 3e-5)
    ctx.assemble()
    p = pkg.sequences.pgse(2000, 8000)
    fn, fo = pkg.sequences.profile_samples(p, 200.0)
    ctx.set_schedule(fn, fo, 200.0)
    q = pkg.sequences.b_to_q(2000.0, p.int4gb())
    return ctx, q, (xyz, tets, reg, fn, fo)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_wait_timeout_is_reported_and_context_recovers(pkg, lib, precision):
    ctx, q, _ = _setup(pkg)
    prec = pkg.PRECISION_FP64 if precision == "fp64" else pkg.PRECISION_MIXED
    rtol = 1e-12 if precision == "fp64" else 1e-9
    g = [0.0, 1.0, 0.0]
    before = ctx.solve([q], g, precision=prec, rtol=rtol)["signal"][0]
    ctx.set_option("wait.limit_ns", 1e6)                 # 1 ms
    ctx.set_option("test.stall_first_wait", 1)
    for _ in range(2):                                    # twice: the context survives each time-out
        with pytest.raises(pkg.BtError) as e:
            ctx.solve([q], g, precision=prec, rtol=rtol)
        assert e.value.code == BT_ERR_TIMEOUT, str(e.value)
        assert "ran out of time" in str(e.value)
    ctx.set_option("test.stall_first_wait", 0)
    ctx.set_option("wait.limit_ns", 2e9)                  # the default
    after = ctx.solve([q], g, precision=prec, rtol=rtol)["signal"][0]
    assert after == before
    ctx.close()


def test_bad_wait_limit_rejected(pkg, lib):
    ctx, _, _ = _setup(pkg)
    for v in (0.0, 10.0, 1e12, float("nan")):
        with pytest.raises(pkg.BtError) as e:
            ctx.set_option("wait.limit_ns", v)
        assert e.value.code == BT_ERR_INVALID
    ctx.close()


def test_invalid_inputs_rejected(pkg, lib):
    ctx, q, (xyz, tets, reg, fn, fo) = _setup(pkg)
    nan, g = float("nan"), [0.0, 1.0, 0.0]
    kp_asym = np.array([[0.0, 1e-5], [2e-5, 0.0]])
    bad_coeffs = [
        ([nan, 3e-3], None, 3e-5), ([-1e-3, 3e-3], None, 3e-5), ([3e-3, 3e-3], [nan, 0.0], 3e-5),
        ([3e-3, 3e-3], [-1e-5, 0.0], 3e-5), ([3e-3, 3e-3], None, nan), ([3e-3, 3e-3], None, -1e-5),
        ([3e-3, 3e-3], None, kp_asym), ([float("inf"), 3e-3], None, 3e-5),
    ]
    for D, iT2, kp in bad_coeffs:
        with pytest.raises(pkg.BtError) as e:
            ctx.set_coefficients(D, iT2, kp)
        assert e.value.code == BT_ERR_INVALID, (D, iT2, kp)
    n_t = len(tets)
    D6 = np.tile([3e-3, 3e-3, 3e-3, 0.0, 0.0, 0.0], (n_t, 1))
    D6[5, 1] = nan
    with pytest.raises(pkg.BtError) as e:
        ctx.set_cell_diffusion(D6)
    assert e.value.code == BT_ERR_INVALID
    iT2c = np.zeros(n_t)
    iT2c[3] = -1e-5
    with pytest.raises(pkg.BtError) as e:
        ctx.set_cell_T2(iT2c)
    assert e.value.code == BT_ERR_INVALID
    fbad = fn.copy()
    fbad[7] = nan
    for args in ((fbad, fo, 200.0), (fn, fo, -200.0), (fn, fo, 0.0), (fn, fo, nan)):
        with pytest.raises(pkg.BtError) as e:
            ctx.set_schedule(*args)
        assert e.value.code == BT_ERR_INVALID
    with pytest.raises(pkg.BtError) as e:
        ctx.set_schedule(fn, fo, 200.0, theta=0.0)
    assert e.value.code == BT_ERR_INVALID
    for qq, gg in ((nan, g), (q, [nan, 1.0, 0.0]), (float("inf"), g)):
        with pytest.raises(pkg.BtError) as e:
            ctx.solve([qq], gg)
        assert e.value.code == BT_ERR_INVALID
    u0 = np.ones(len(xyz))
    u0[2] = nan
    with pytest.raises(pkg.BtError) as e:
        ctx.solve([q], g, u0=u0)
    assert e.value.code == BT_ERR_INVALID
    for rt, mi in ((0.0, 100), (-1e-9, 100), (nan, 100), (1e-9, 0)):
        with pytest.raises(pkg.BtError) as e:
            ctx.solve([q], g, rtol=rt, max_iterations=mi)
        assert e.value.code == BT_ERR_INVALID
    # nothing above changed the context: the original coefficients and schedule still solve
    ctx.set_schedule(fn, fo, 200.0)
    out = ctx.solve([q], g, rtol=1e-12)
    assert 0.0 < out["signal"][0] / out["S0"] < 1.0
    ctx.close()


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_iteration_cap_reports_not_converged(pkg, lib, precision):
    ctx, q, _ = _setup(pkg)
    prec = pkg.PRECISION_FP64 if precision == "fp64" else pkg.PRECISION_MIXED
    with pytest.raises(pkg.BtError) as e:
        ctx.solve([q], [0.0, 1.0, 0.0], precision=prec, rtol=1e-12 if precision == "fp64" else 1e-9,
                  max_iterations=1)
    assert e.value.code == BT_ERR_NOT_CONVERGED, str(e.value)
    out = ctx.solve([q], [0.0, 1.0, 0.0], precision=prec, rtol=1e-9, max_iterations=5000)
    assert 0.0 < out["signal"][0] / out["S0"] < 1.0
    ctx.close()
