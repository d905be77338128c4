"""torch.autograd.Function over the GPU adjoint gradient.

``circuit_loss(circuit, params, weights)`` returns
L = sum_q w_q <Z_q> of the circuit run from |0...0> with its RX/RY/RZ angles
set to ``params`` (Circuit.set_parameters order). The forward runs the
circuit and the exact <Z_q> reduction only. The gradient with respect to the
angles is computed in ``backward``, and only when autograd asks for it, by the
adjoint sweep of libdamavand_gpu: one forward plus one reverse pass that
uncomputes the state, with the per-parameter Im<lambda|P|psi> reductions
fused into the sweep, instead of 2P parameter-shift forwards. dL/dw_q is the
exact <Z_q> saved by the forward.

Tensors may live on any device; results come back on the device (and in the
dtype) of the tensor they belong to. The angles always cross to the host once
per call: the gate matrices are formed on the host with the same libm calls as
the reference's gate formulas (src/qubit_backend/gates.rs), so that every
arithmetic starts from identical coefficients. <Z_q> (n values) and the
gradients (one per angle) come back from the library as host arrays.
"""
from __future__ import annotations

import numpy as np
import torch


class CircuitExpectation(torch.autograd.Function):
    @staticmethod
    def forward(ctx, params: torch.Tensor, weights: torch.Tensor, circuit):
        p = params.detach().to("cpu", torch.float64).numpy().copy()
        circuit.set_parameters(p)
        circuit.reset_amplitudes()
        circuit.forward()
        ez = torch.from_numpy(np.asarray(circuit.expectation_z(), dtype=np.float64)).to(weights.device)
        loss = torch.dot(weights.detach().to(torch.float64), ez)
        ctx.circuit = circuit
        ctx.params = p
        ctx.save_for_backward(weights.detach(), ez)
        ctx.param_meta = (params.device, params.dtype)
        return loss.to(device=params.device, dtype=params.dtype)

    @staticmethod
    def backward(ctx, grad_out):
        weights, ez = ctx.saved_tensors
        gp = gw = None
        if ctx.needs_input_grad[0]:
            w = weights.to("cpu", torch.float64).numpy()
            ctx.circuit.set_parameters(ctx.params)
            _, grads = ctx.circuit.adjoint_gradient(w)
            dev, dt = ctx.param_meta
            g = torch.from_numpy(np.asarray(grads, dtype=np.float64)).to(dev)
            gp = (grad_out.detach().to(dev, torch.float64) * g).to(dt)
        if ctx.needs_input_grad[1]:
            gw = (grad_out.detach().to(ez.device, torch.float64) * ez).to(weights.dtype)
        return gp, gw, None


def circuit_loss(circuit, params: torch.Tensor, weights: torch.Tensor) -> torch.Tensor:
    return CircuitExpectation.apply(params, weights, circuit)
