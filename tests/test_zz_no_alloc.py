"""bt_signal_noalloc: the allocation-free signal readout.

Callers that cannot allocate device memory when they read a signal (code inside
CUDA stream capture, serving or acquisition threads with a frozen allocator)
use this entry point; it keeps its scratch in a static device array.  The tests
call it through the C ABI and compare it with an independent host FP64 sum
(np.dot(w, Re u)) and with the signal the regular entry point (bt_solve)
returns for the same state, on two calls in a row, within the FP64 parity
tolerance used by the other GPU tests; they also run it at the largest size its
scratch allows (2,097,152 dofs), at a size that is not a multiple of its
2,048-element block, and check that a size one beyond the limit is rejected.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-9
MAX_N = 2097152           # 1024 blocks x 2048 elements of static scratch


def _call(lib, d_w, d_u, n, d_sig, stream):
    return lib.bt_signal_noalloc(ctypes.c_void_p(d_w.data_ptr()), ctypes.c_void_p(d_u.data_ptr()), int(n),
                                 ctypes.c_void_p(d_sig.data_ptr()), ctypes.c_void_p(stream))


def test_signal_noalloc_matches_solve(pkg, lib):
    import torch
    xyz, tets = pkg.meshgen.kuhn_box(-6, 6, 8)
    reg = pkg.meshgen.cylinder_regions(xyz, tets, [(0.5, 0.0)], [3.5])
    prof = pkg.sequences.pgse(2000, 8000)
    fn, fo = pkg.sequences.profile_samples(prof, 200.0)
    ctx = pkg.Context(0)
    ctx.mesh_upload(xyz, tets, reg, 2)
    ctx.set_coefficients([3e-3, 2e-3], None, 3e-5)
    ctx.assemble()
    ctx.set_schedule(fn, fo, 200.0)
    q = [pkg.sequences.b_to_q(b, prof.int4gb()) for b in (1500.0, 3000.0)]
    out = ctx.solve(q, [[0.0, 1.0, 0.0], [0.6, 0.0, 0.8]], rtol=1e-12)
    _, _, w = ctx.dofs()
    n = len(w)
    dev = torch.device("cuda", 0)
    d_w = torch.tensor(w, dtype=torch.float64, device=dev)
    d_sig = torch.zeros(1, dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream(dev).cuda_stream
    for k in range(2):                       # two calls in a row share the scratch
        u = ctx.solution(k)
        d_u = torch.tensor(np.stack([u.real, u.imag], axis=1).ravel(), dtype=torch.float64, device=dev)
        d_sig.fill_(float("nan"))
        torch.cuda.synchronize()
        assert _call(lib, d_w, d_u, n, d_sig, stream) == 0
        torch.cuda.synchronize()
        got = float(d_sig.cpu()[0])
        host = float(np.dot(w, u.real))      # independent FP64 sum on the host
        assert abs(got - host) <= SIG_RTOL * abs(host), (k, got, host)
        ref = float(out["signal"][k])
        assert abs(got - ref) <= SIG_RTOL * abs(ref), (k, got, ref)
    ctx.close()


def test_signal_noalloc_size_limits(lib):
    import torch
    dev = torch.device("cuda", 0)
    stream = torch.cuda.current_stream(dev).cuda_stream
    rng = np.random.default_rng(7)
    w = rng.uniform(0.5, 1.5, MAX_N)
    u = rng.uniform(0.1, 1.0, 2 * MAX_N)     # (re, im) pairs; all products positive: no cancellation
    d_w = torch.tensor(w, dtype=torch.float64, device=dev)
    d_u = torch.tensor(u, dtype=torch.float64, device=dev)
    d_sig = torch.zeros(1, dtype=torch.float64, device=dev)
    for n in (MAX_N, MAX_N - 777, 1):        # the limit, a ragged size, one element
        for _ in range(2):                   # two calls in a row
            d_sig.fill_(float("nan"))
            torch.cuda.synchronize()
            assert _call(lib, d_w, d_u, n, d_sig, stream) == 0
            torch.cuda.synchronize()
            got = float(d_sig.cpu()[0])
            host = float(np.dot(w[:n], u[0:2 * n:2]))
            assert abs(got - host) <= 1e-12 * abs(host), (n, got, host)
    # sizes beyond the static scratch, and empty input, are rejected with no work queued
    assert _call(lib, d_w, d_u, MAX_N + 1, d_sig, stream) == 1
    assert _call(lib, d_w, d_u, 0, d_sig, stream) == 1
