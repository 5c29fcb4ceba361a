"""torch.autograd bridge for the whole-step reverse mode.

``StepLoss.apply(xp, qp, vpm, nsteps, dt, probes, ke_weight)`` returns the
scalar loss of ``nsteps`` particle-mesh steps (field step, Euler push,
remesh) from particles ``xp`` (NVR, 3) and ``qp`` (NVR, 4) -- the
reference's XP / QP layout -- and back-propagates d loss / d xp and
d loss / d qp[:, :3] computed by the library's exact transpose of every
step (``vpmg_adjoint_run``).  QP(4) (the particle volume) is treated as a
constant.  The library computes on the GPU in the handle's arithmetic
(IEEE FP64 unless the handle was set to float-float); the tensors may live
on any device and are copied through host memory.
"""
import numpy as np
import torch


class StepLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, xp, qp, vpm, nsteps, dt, probes=None, ke_weight=0.0):
        x = xp.detach().to("cpu", torch.float64).contiguous().numpy()
        q = qp.detach().to("cpu", torch.float64).contiguous().numpy()
        vpm.set_particles(x, q)
        pr = None if probes is None else np.asarray(probes, dtype=np.float64)
        loss, xbar, qbar, _, _ = vpm.adjoint_run(nsteps, dt, pr, ke_weight)
        gq = np.zeros_like(q)
        gq[:, :3] = qbar
        ctx.save_for_backward(torch.from_numpy(xbar).to(xp.device, xp.dtype), torch.from_numpy(gq).to(qp.device, qp.dtype))
        return torch.tensor(loss, dtype=xp.dtype, device=xp.device)

    @staticmethod
    def backward(ctx, g):
        gx, gq = ctx.saved_tensors
        return g * gx, g * gq, None, None, None, None, None
