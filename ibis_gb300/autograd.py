"""torch.autograd wrapper of the residual: R(U) = dU/dt of a Simulation as a
differentiable function of the conserved state, with the hand-written tangent
(forward mode) and adjoint (reverse mode) kernels as its derivatives.

    from ibis_gb300.autograd import residual
    U = torch.tensor(sim.conserved(), device="cuda", requires_grad=True)
    R = residual(sim, U)              # FiniteVolume::compute_dudt, FP64
    (R * w).sum().backward()          # U.grad = (dR/dU)^T w, ibisgb_vjp_device

The forward pass evaluates the residual in the FP64_EXACT build (the
reference's operation order), so the backward pass is the exact transpose of
the derivative of what forward returned.  Both run on the current CUDA stream.
"""
from __future__ import annotations

import torch


class Residual(torch.autograd.Function):
    @staticmethod
    def forward(ctx, U, sim):
        if U.dtype != torch.float64 or not U.is_cuda:
            raise TypeError("U must be a float64 CUDA tensor")
        U = U.contiguous()
        stream = torch.cuda.current_stream()
        sim.set_conserved_into(U, stream=stream)
        out = torch.empty_like(U)
        sim.compute_dudt_into(out, "f64_exact", stream=stream)
        ctx.sim = sim
        ctx.save_for_backward(U)
        ctx.save_for_forward(U)
        return out

    @staticmethod
    def backward(ctx, grad_out):
        (U,) = ctx.saved_tensors
        sim = ctx.sim
        stream = torch.cuda.current_stream()
        sim.set_conserved_into(U, stream=stream)  # linearise at the forward state
        g = torch.empty_like(U)
        sim.vector_jacobian_product_into(grad_out.contiguous(), g, stream=stream)
        return g, None

    @staticmethod
    def jvp(ctx, dU, _):
        (U,) = ctx.saved_tensors
        sim = ctx.sim
        stream = torch.cuda.current_stream()
        sim.set_conserved_into(U, stream=stream)
        out = torch.empty_like(U)
        sim.matrix_vector_product_into(dU.contiguous(), out, inv_dt_star=0.0, stream=stream)
        return -out  # matrix_vector_product gives inv_dt v - J v


def residual(sim, U):
    """dU/dt of `sim` at conserved state U (float64 CUDA tensor, N x n_conserved)."""
    return Residual.apply(U, sim)
