"""torch.autograd.Function over the engine's discrete adjoint.

``BlochTorreySignal.apply(D, invT2, kappa, engine, q, gdir, sequence)`` returns
the normalised signal S/S0 of one FP64 solve as a 0-d tensor; its backward
returns dS/dD (per region), dS/d(1/T2) (per region) and dS/dkappa (per region
pair, symmetric matrix), computed by ``bt_adjoint`` during the forward call
(one forward sweep, one checkpointed backward sweep).  Tensors live on the
host: they are the tissue parameters, not the field.
"""

import numpy as np
import torch


class BlochTorreySignal(torch.autograd.Function):
    @staticmethod
    def forward(ctx, D, invT2, kappa, engine, q, gdir, sequence=0):
        Dn = D.detach().cpu().double().numpy()
        Tn = invT2.detach().cpu().double().numpy()
        Kn = kappa.detach().cpu().double().numpy()
        engine.set_coefficients(Dn, Tn, Kn)
        engine.assemble()
        out = engine.adjoint(q, gdir, sequence)
        S0 = engine.info()["volume"]
        ctx.save_for_backward(torch.from_numpy(out["dD"] / S0), torch.from_numpy(out["dinvT2"] / S0),
                              torch.from_numpy(out["dkappa"] / S0))
        return torch.tensor(out["signal"] / S0, dtype=torch.float64)

    @staticmethod
    def backward(ctx, grad):
        gD, gT, gK = ctx.saved_tensors
        return grad * gD, grad * gT, grad * gK, None, None, None, None
