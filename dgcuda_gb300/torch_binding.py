"""torch.autograd.Function over the C ABI's discrete adjoint (the only use
of PyTorch in the package; a thin test binding).

    h_samples = DGShallowWater.apply(h0, b, adjoint, nsteps, dt, every, ckpt)

h0: initial water height modes [mode][elem] (float64 tensor), b: bed modes
[mode][elem]; the momenta are taken from the solver's state at call time.
Returns the receiver samples [nsamp][nrec].  backward() runs the
checkpointed reverse sweep (dg_adjoint_backward) and returns d/dh0, d/db.
"""
import numpy as np
import torch


class DGShallowWater(torch.autograd.Function):
    @staticmethod
    def forward(ctx, h0, b, adjoint, nsteps, dt, every, ckpt):
        s = adjoint.solver
        c = s.get_state()
        c[0] = h0.detach().cpu().numpy().reshape(s.n_p, s.K)
        s.set_state(c)
        s.set_bathymetry(b.detach().cpu().numpy().reshape(s.n_p, s.K))
        samples = adjoint.forward(nsteps, dt, every, ckpt)
        ctx.adjoint = adjoint
        ctx.shape_h, ctx.shape_b = h0.shape, b.shape
        return torch.from_numpy(np.ascontiguousarray(samples))

    @staticmethod
    def backward(ctx, gsamples):
        gu, gb = ctx.adjoint.backward(gsamples.detach().cpu().numpy())
        return (torch.from_numpy(gu[0].copy()).reshape(ctx.shape_h),
                torch.from_numpy(gb).reshape(ctx.shape_b), None, None, None, None, None)
