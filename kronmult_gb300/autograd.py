"""torch.autograd wrapper over the C ABI, used to check the adjoint kernel.

`KronmultFunction.apply(factors, inputs, spec)` returns the (n_out, N) outputs
out[e] = sum_{k: out_index[k] = e} kron(A_k) . inputs[k]; its backward is the
hand-written adjoint kernel (kronmult_batched_adjoint_*).  This wrapper exists so
that the adjoint can be checked against finite differences and against the
reference applied with transposed factors; it is not a training framework.
"""
from __future__ import annotations

from dataclasses import dataclass

import torch

from .api import DeviceBatch, adjoint


@dataclass(frozen=True)
class KronSpec:
    d: int
    n: int
    stride: int
    n_out: int
    fac_index: torch.Tensor
    out_index: torch.Tensor


class KronmultFunction(torch.autograd.Function):
    @staticmethod
    def forward(ctx, factors: torch.Tensor, inputs: torch.Tensor, spec: KronSpec):
        factors = factors.contiguous()
        inputs = inputs.contiguous()
        out = torch.zeros((spec.n_out, spec.n ** spec.d), dtype=inputs.dtype, device=inputs.device)
        b = DeviceBatch(spec.d, spec.n, spec.stride, factors, inputs, out, spec.fac_index, spec.out_index)
        b.forward()
        ctx.save_for_backward(factors, inputs)
        ctx.spec = spec
        return out

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        factors, inputs = ctx.saved_tensors
        spec = ctx.spec
        b = DeviceBatch(spec.d, spec.n, spec.stride, factors, inputs,
                        torch.empty((spec.n_out, spec.n ** spec.d), dtype=inputs.dtype, device=inputs.device),
                        spec.fac_index, spec.out_index)
        gin = torch.zeros_like(inputs) if ctx.needs_input_grad[1] else None
        gfac = torch.zeros_like(factors) if ctx.needs_input_grad[0] else None
        if gin is not None or gfac is not None:
            adjoint(b, grad_out.contiguous(), gin, gfac)
        return gfac, gin, None


def kronmult(factors: torch.Tensor, inputs: torch.Tensor, spec: KronSpec) -> torch.Tensor:
    return KronmultFunction.apply(factors, inputs, spec)
