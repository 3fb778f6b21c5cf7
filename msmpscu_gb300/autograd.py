"""torch.autograd wrappers of the differentiation kernels (test harness).

``EAMForce``: forward = the library's force call, backward = J^T g with J = dF/dx = -H; the
Hessian of a conservative force field is symmetric, so J^T g = -H g is one HVP call.  (For
tabulated potentials the pair-force and density tables are interpolated independently and
the Jacobian is symmetric only up to the table interpolation error, ~1e-6 relative.)
``ForceMatchLoss``: forward = sum |F(theta) - F_target|^2 over all boxes of the engine,
backward = the adjoint kernel's dL/dtheta for theta = (A, xi, p, q, r0).
Tensors are float64 on the CPU; every evaluation goes through the C ABI.
"""
import numpy as np
import torch

from . import _lib as L
from .engine import ForceTable


class EAMForce(torch.autograd.Function):
    @staticmethod
    def forward(ctx, x, engine, boxes):
        engine.copyin(boxes, x.detach().numpy())
        engine.calforce()
        ctx.engine, ctx.boxes = engine, boxes
        ctx.save_for_backward(x)
        return torch.from_numpy(engine.get_force())

    @staticmethod
    def backward(ctx, g):
        (x,) = ctx.saved_tensors
        e = ctx.engine
        e.copyin(ctx.boxes, x.detach().numpy())
        hv = e.hvp(g.detach().numpy())
        return torch.from_numpy(-hv), None, None


class ForceMatchLoss(torch.autograd.Function):
    @staticmethod
    def forward(ctx, theta, engine, ftarget, rc):
        prm = theta.detach().numpy().astype(np.float64)
        engine.init_forcetable(ForceTable(L.POT_CR, prm, rc, rc, L.FS_TYPE))
        loss, grad = engine.param_adjoint(prm, ftarget)
        ctx.save_for_backward(torch.from_numpy(grad))
        return torch.tensor(loss, dtype=torch.float64)

    @staticmethod
    def backward(ctx, gl):
        (grad,) = ctx.saved_tensors
        return gl * grad, None, None, None
