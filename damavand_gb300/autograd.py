"""torch.autograd.Function over the GPU adjoint gradient.

``circuit_loss(circuit, params, weights)`` returns
L = sum_q w_q <Z_q> of the circuit run from |0...0> with its RX/RY/RZ angles
set to ``params`` (Circuit.set_parameters order). Its backward uses the
adjoint sweep of libdamavand_gpu (one forward plus one reverse pass that
uncomputes the state, with the per-parameter Im<lambda|P|psi> reductions
fused into the sweep) instead of 2P parameter-shift forwards. dL/dw_q is the
exact <Z_q>.
"""
from __future__ import annotations

import numpy as np
import torch


class CircuitExpectation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, weights: torch.Tensor, circuit):
        p = params.detach().to("cpu", torch.float64).numpy()
        w = weights.detach().to("cpu", torch.float64).numpy()
        circuit.set_parameters(p)
        if params.requires_grad:
            loss, grads = circuit.adjoint_gradient(w)
        else:
            loss, grads = circuit.loss(w), np.zeros(p.size)
        ez = circuit.expectation_z()  # state holds the forward state in both branches
        ctx.save_for_backward(torch.from_numpy(np.asarray(grads, dtype=np.float64)),
                              torch.from_numpy(np.asarray(ez, dtype=np.float64)))
        ctx.devices = (params.device, weights.device)
        ctx.dtypes = (params.dtype, weights.dtype)
        return torch.tensor(loss, dtype=params.dtype, device=params.device)

    @staticmethod
    def backward(ctx, grad_out):
        grads, ez = ctx.saved_tensors
        g = grad_out.detach().to("cpu", torch.float64)
        gp = (g * grads).to(ctx.devices[0], ctx.dtypes[0])
        gw = (g * ez).to(ctx.devices[1], ctx.dtypes[1])
        return gp, gw, None


def circuit_loss(circuit, params: torch.Tensor, weights: torch.Tensor) -> torch.Tensor:
    return CircuitExpectation.apply(params, weights, circuit)
