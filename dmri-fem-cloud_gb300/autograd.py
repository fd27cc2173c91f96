"""torch.autograd.Functions over the engine's discrete adjoints.

``BlochTorreySignal.apply(D, invT2, kappa, engine, q, gdir, sequence)`` returns
the normalised signal S/S0 of one FP64 solve as a 0-d tensor; its backward
returns dS/dD (per region), dS/d(1/T2) (per region) and dS/dkappa (per region
pair, symmetric matrix), computed by ``bt_adjoint`` during the forward call
(one forward sweep, one checkpointed backward sweep).

``BlochTorreySignals.apply(D, invT2, kappa, engine, q[n], gdir[n, 3],
sequence[n] or None)`` does the same for n signals at once through the batched
mixed-precision adjoint (``bt_adjoint_batch``: the signals advance together,
forward and backward): it returns the n normalised signals, and its backward
contracts the incoming gradient with the n per-signal derivatives.

``BlochTorreyCellField.apply(D_cell[n_cells, 6], invT2_cell[n_cells], engine, q,
gdir, sequence)`` is the field form: a per-cell diffusion tensor (xx, yy, zz,
xy, xz, yz) and a per-cell 1/T2 go into the FP64 solve, and the backward
returns dS/dD_cell and dS/d(1/T2)_cell from ``bt_adjoint_cells`` (for fitting
a diffusivity or relaxation map).

``BlochTorreyCellFields.apply(D_cell, invT2_cell, engine, q[n], gdir[n, 3],
sequence[n] or None)`` returns n normalised signals of the mixed-precision
batched solve with those fields; its backward runs the batched adjoint once with
the incoming gradient as signal weights (``bt_adjoint_batch_cells``) and returns
the per-cell gradients.

The tissue parameters may be CPU or CUDA tensors of any floating dtype; they
are read on the host and the gradients are returned on the parameters' own
device and dtype.
"""

import numpy as np
import torch


def _host(t):
    return t.detach().to("cpu", torch.float64).numpy()


class BlochTorreySignal(torch.autograd.Function):
    @staticmethod
    def forward(ctx, D, invT2, kappa, engine, q, gdir, sequence=0):
        engine.set_coefficients(_host(D), _host(invT2), _host(kappa))
        engine.assemble()
        out = engine.adjoint(q, gdir, sequence)
        S0 = engine.info()["volume"]
        ctx.like = [(x.device, x.dtype) for x in (D, invT2, kappa)]
        ctx.save_for_backward(torch.from_numpy(out["dD"] / S0), torch.from_numpy(out["dinvT2"] / S0),
                              torch.from_numpy(out["dkappa"] / S0))
        return torch.tensor(out["signal"] / S0, dtype=D.dtype, device=D.device)

    @staticmethod
    def backward(ctx, grad):
        g = float(grad.detach().to("cpu", torch.float64))
        outs = [(g * t).to(dev, dt) for t, (dev, dt) in zip(ctx.saved_tensors, ctx.like)]
        return outs[0], outs[1], outs[2], None, None, None, None


class BlochTorreySignals(torch.autograd.Function):
    @staticmethod
    def forward(ctx, D, invT2, kappa, engine, q, gdir, sequence=None):
        engine.set_coefficients(_host(D), _host(invT2), _host(kappa))
        engine.assemble()
        out = engine.adjoint_batch(np.asarray(q, np.float64), np.asarray(gdir, np.float64), sequence)
        S0 = engine.info()["volume"]
        ctx.like = [(x.device, x.dtype) for x in (D, invT2, kappa)]
        ctx.save_for_backward(torch.from_numpy(out["dD"] / S0), torch.from_numpy(out["dinvT2"] / S0),
                              torch.from_numpy(out["dkappa"] / S0))
        return torch.from_numpy(out["signal"] / S0).to(D.device, D.dtype)

    @staticmethod
    def backward(ctx, grad):
        g = grad.detach().to("cpu", torch.float64)          # [n]
        gD, gT, gK = ctx.saved_tensors                      # [n, nr], [n, nr], [n, nr, nr]
        outs = [torch.tensordot(g, t, dims=1) for t in (gD, gT, gK)]
        outs = [t.to(dev, dt) for t, (dev, dt) in zip(outs, ctx.like)]
        return outs[0], outs[1], outs[2], None, None, None, None


class BlochTorreyCellField(torch.autograd.Function):
    @staticmethod
    def forward(ctx, D_cell, invT2_cell, engine, q, gdir, sequence=0):
        engine.set_cell_diffusion(np.ascontiguousarray(_host(D_cell).reshape(-1, 6)))
        engine.set_cell_T2(np.ascontiguousarray(_host(invT2_cell).reshape(-1)))
        engine.assemble()
        out = engine.adjoint_cells(q, gdir, sequence)
        S0 = engine.info()["volume"]
        ctx.like = [(x.device, x.dtype) for x in (D_cell, invT2_cell)]
        ctx.save_for_backward(torch.from_numpy(out["dD_cell"] / S0), torch.from_numpy(out["dinvT2_cell"] / S0))
        return torch.tensor(out["signal"] / S0, dtype=D_cell.dtype, device=D_cell.device)

    @staticmethod
    def backward(ctx, grad):
        g = float(grad.detach().to("cpu", torch.float64))
        gD, gT = ctx.saved_tensors                          # [n_cells, 6], [n_cells]
        (dD, tD), (dT, tT) = ctx.like
        return (g * gD).to(dD, tD), (g * gT).to(dT, tT), None, None, None, None


class BlochTorreyCellFields(torch.autograd.Function):
    @staticmethod
    def forward(ctx, D_cell, invT2_cell, engine, q, gdir, sequence=None):
        engine.set_cell_diffusion(np.ascontiguousarray(_host(D_cell).reshape(-1, 6)))
        engine.set_cell_T2(np.ascontiguousarray(_host(invT2_cell).reshape(-1)))
        engine.assemble()
        q = np.atleast_1d(np.asarray(q, np.float64))
        gdir = np.asarray(gdir, np.float64).reshape(len(q), 3)
        out = engine.solve(q, gdir, sequence, None, 1, 1e-9, 20000)     # mixed precision
        S0 = engine.info()["volume"]
        ctx.engine, ctx.q, ctx.gdir, ctx.sequence, ctx.S0 = engine, q, gdir, sequence, S0
        ctx.like = [(x.device, x.dtype) for x in (D_cell, invT2_cell)]
        return torch.from_numpy(out["signal"] / S0).to(D_cell.device, D_cell.dtype)

    @staticmethod
    def backward(ctx, grad):
        w = grad.detach().to("cpu", torch.float64).numpy() / ctx.S0
        out = ctx.engine.adjoint_batch_cells(ctx.q, ctx.gdir, w, ctx.sequence)
        (dD, tD), (dT, tT) = ctx.like
        return (torch.from_numpy(out["dD_cell"]).to(dD, tD), torch.from_numpy(out["dinvT2_cell"]).to(dT, tT),
                None, None, None, None)
