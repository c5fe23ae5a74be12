"""PyTorch layer: the L2 waveform misfit of a medium (vp, vs, rho) as a
differentiable function, for use inside torch optimisers and models.

    import psvwave_gb300 as psv
    from psvwave_gb300.torch_ops import l2_misfit

    model = psv.fdModel("configuration.ini")
    model.set_observed_data(ux_obs, uz_obs)
    vp = torch.tensor(vp0, device="cuda", requires_grad=True)  # likewise vs, rho
    chi = l2_misfit(model, vp, vs, rho, checkpoint_every=100)
    chi.backward()            # vp.grad, vs.grad, rho.grad

The misfit is the reference's calculate_l2_misfit over all shots
(src/fdModel.cpp:1128-1145). Two gradients are available:

* mode="exact" (default): the exact discrete adjoint, i.e. the transpose of
  the solver's time stepping. It is the gradient of the computed misfit,
  which central finite differences confirm. Forward states are rebuilt from
  checkpoints taken every `checkpoint_every` steps; checkpoint_every = nt
  keeps every state instead.
* mode="reference": the reference's own adjoint kernels (run_model,
  src/fdModel.cpp:1291-1308: forward with snapshots, adjoint sources,
  reverse-time adjoint, map_kernels_to_velocity). This is a continuous-adjoint
  approximation that correlates snapshots every snapshot_interval steps over
  the free region, so it only points the same way as the exact gradient.

The gradient is computed together with the misfit whenever an input requires
grad (the forward run is part of it); with no input requiring grad only the
forward runs and the misfit are computed. Inputs may be CUDA tensors on the
model's device (no host round trip) or CPU tensors. The function has no
double backward.
"""
import numpy as np
import torch

__all__ = ["L2Misfit", "l2_misfit"]


def _set_medium(model, vp, vs, rho):
    if vp.is_cuda:
        model.set_parameter_fields_device(vp, vs, rho)
    else:
        model.set_parameter_fields(*(t.detach().to(torch.float64).numpy() for t in (vp, vs, rho)))


def _misfit_only(model):
    for shot in range(model.n_shots):
        model.forward_simulate(shot, False)
    model.calculate_l2_misfit()
    return model.misfit


class L2Misfit(torch.autograd.Function):
    """apply(vp, vs, rho, model, checkpoint_every, mode) -> misfit (float64
    scalar on vp's device). Gradients flow to vp, vs and rho."""

    @staticmethod
    def forward(ctx, vp, vs, rho, model, checkpoint_every, mode):
        if mode not in ("exact", "reference"):
            raise ValueError("mode must be 'exact' or 'reference'")
        _set_medium(model, vp, vs, rho)
        dev = vp.device
        if not any(ctx.needs_input_grad[:3]):
            return torch.tensor(_misfit_only(model), dtype=torch.float64, device=dev)
        if mode == "exact":
            if vp.is_cuda:
                misfit, grads = model.exact_gradient(checkpoint_every, on_device=True)
            else:
                misfit, g = model.exact_gradient(checkpoint_every)
                grads = tuple(torch.from_numpy(np.ascontiguousarray(a)) for a in g)
        else:
            model.compute_gradients()
            misfit = model.misfit
            if vp.is_cuda:
                grads = model.get_kernels_device()
            else:
                grads = tuple(torch.from_numpy(a) for a in model.get_kernels())
        grads = tuple(g.to(dtype=t.dtype) for g, t in zip(grads, (vp, vs, rho)))
        ctx.save_for_backward(*grads)
        return torch.tensor(misfit, dtype=torch.float64, device=dev)

    @staticmethod
    def backward(ctx, grad_out):
        g_vp, g_vs, g_rho = ctx.saved_tensors
        scale = grad_out.to(g_vp.dtype)
        return (scale * g_vp if ctx.needs_input_grad[0] else None,
                scale * g_vs if ctx.needs_input_grad[1] else None,
                scale * g_rho if ctx.needs_input_grad[2] else None, None, None, None)


def l2_misfit(model, vp, vs, rho, checkpoint_every=100, mode="exact"):
    """The L2 misfit of `model`'s observed data against synthetics of the
    medium (vp, vs, rho) ([nx, nz] tensors), differentiable in the medium."""
    return L2Misfit.apply(vp, vs, rho, model, int(checkpoint_every), mode)
