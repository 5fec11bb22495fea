"""torch.autograd face of the engine (the differentiation form).

``DFJK.apply(C, B)`` returns (J, K) for the lr-symmetric density C C^T; its backward calls the
engine's hand-written reverse kernels (``gdfjk_backward``), which recompute (Q|mi) instead of
storing it, and return dE/dC and — when ``B`` requires grad — dE/dB, the B-space 3-index
density that psi4 contracts with derivative integrals (jk_grad.cc:294-832).  ``B`` is the
Q-major packed triangle the engine holds (naux x nbf(nbf+1)/2); it is only a handle for the
gradient — the forward reads the engine's resident copy.
"""
from __future__ import annotations

import torch

from . import _jkabi as abi


class DFJK(torch.autograd.Function):
    @staticmethod
    def forward(ctx, C, B, engine):
        if C.dtype != torch.float64 or not C.is_cuda:
            raise TypeError("C must be a float64 CUDA tensor")
        C = C.contiguous()
        nbf, nocc = C.shape
        J = torch.empty((nbf, nbf), dtype=torch.float64, device=C.device)
        K = torch.empty_like(J)
        torch.cuda.current_stream(C.device).synchronize()
        engine.compute_device(C.data_ptr(), None, nocc, max(nocc, 1), abi.DO_J | abi.DO_K, None, J.data_ptr(), K.data_ptr())
        engine.synchronize()
        ctx.save_for_backward(C)
        ctx.engine = engine
        ctx.want_B = B is not None and B.requires_grad
        ctx.B_shape = None if B is None else B.shape
        return J, K

    @staticmethod
    def backward(ctx, gJ, gK):
        (C,) = ctx.saved_tensors
        eng = ctx.engine
        nbf, nocc = C.shape
        gJ = torch.zeros((nbf, nbf), dtype=torch.float64, device=C.device) if gJ is None else gJ.contiguous()
        gK = torch.zeros((nbf, nbf), dtype=torch.float64, device=C.device) if gK is None else gK.contiguous()
        dC = torch.empty_like(C) if ctx.needs_input_grad[0] else None
        G = torch.empty(ctx.B_shape, dtype=torch.float64, device=C.device) if ctx.want_B else None
        torch.cuda.current_stream(C.device).synchronize()
        eng.backward_device(C.data_ptr(), nocc, max(nocc, 1), gJ.data_ptr(), gK.data_ptr(),
                            None if dC is None else dC.data_ptr(), None if G is None else G.data_ptr())
        eng.synchronize()
        return dC, G, None
