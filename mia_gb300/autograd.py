"""torch.autograd binding of a level's cost and its adjoint (for tests and
for composing the registration cost with other torch terms).

``level_costs(params, level)`` returns the 2-vector (image cost, penalty
cost) of `level` (a ``mia_gb300.Level`` with its images set) at `params`
(a float64 tensor of level.nparams, CPU or CUDA).  Its backward applies the
gradients that the adjoint kernels compute (warp, adjoint, gather: the
evaluate_fdf path through mgr_level_evaluate):

* d(image cost)/d(params) is the image gradient as the reference computes
  it (the force from central differences of the warped image folded onto
  the coefficients, C3DSplineTransformation::translate);
* d(penalty cost)/d(params) is the negative of the penalty gradient the
  reference returns (its divcurl penalty reports -weight * gradient,
  mia/3d/splinetransformpenalty.cc:52-71), so that the binding gives the
  derivative of the value it returns.
"""
import numpy as np
import torch


class _LevelCosts(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params, level):
        p = params.detach().to("cpu", torch.float64).contiguous().numpy()
        if p.size != level.nparams:
            raise ValueError("params must hold level.nparams values")
        ci, cp, gi, gp, _ = level.evaluate(p)
        ctx.save_for_backward(torch.from_numpy(np.ascontiguousarray(gi)).to(params.device),
                              torch.from_numpy(np.ascontiguousarray(-gp)).to(params.device))
        return torch.tensor([ci, cp], dtype=torch.float64, device=params.device)

    @staticmethod
    def backward(ctx, grad_costs):
        d_image, d_penalty = ctx.saved_tensors
        return grad_costs[0] * d_image + grad_costs[1] * d_penalty, None


def level_costs(params, level):
    """(image cost, penalty cost) of `level` at `params`, differentiable in params"""
    return _LevelCosts.apply(params, level)
