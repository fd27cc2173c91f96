"""bt_signal_noalloc: the allocation-free signal readout.

Callers that cannot allocate device memory when they read a signal (code inside
CUDA stream capture, serving or acquisition threads with a frozen allocator)
use this entry point; it keeps its scratch in a static device array.  The test
checks it through the C ABI against the signal the regular entry point
(bt_solve) returns for the same state, on two calls in a row, within the FP64
parity tolerance used by the other GPU tests.
"""

import ctypes

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

SIG_RTOL = 1e-9


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
        rc = lib.bt_signal_noalloc(ctypes.c_void_p(d_w.data_ptr()), ctypes.c_void_p(d_u.data_ptr()), n,
                                   ctypes.c_void_p(d_sig.data_ptr()), ctypes.c_void_p(stream))
        assert rc == 0
        torch.cuda.synchronize()
        got = float(d_sig.cpu()[0])
        ref = float(out["signal"][k])
        assert abs(got - ref) <= SIG_RTOL * abs(ref), (k, got, ref)
    # sizes beyond the static scratch are rejected, with no work queued
    rc = lib.bt_signal_noalloc(ctypes.c_void_p(d_w.data_ptr()), ctypes.c_void_p(d_u.data_ptr()), 2097153,
                               ctypes.c_void_p(d_sig.data_ptr()), ctypes.c_void_p(stream))
    assert rc == 1
    ctx.close()
