"""torch.autograd.Function over the EP batch loss with the hand-written
backward kernels.

``EPBatchLoss(...)(table, anchors, nbr_ptr, nbr, nbr_w, negatives)`` returns
the per-anchor losses of one batch of explicit samples (roles as in
``src/algos/ep/mod.rs:289-327``) as a differentiable function of the feature
table.  FP32 tables run the training kernels; FP64 tables run the same
kernels instantiated in double precision (used for finite-difference checks
only).  Backward evaluates the forward again with the upstream gradient folded
into the per-role scales, then reduces exactly as training does (sorted,
deterministic) and scatters the touched rows into a dense gradient.
"""
from __future__ import annotations

import torch

from . import _native
from .ep import EPLoss


class _Fn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, table, owner, samples):
        if not table.is_cuda:
            raise ValueError("the table must be a CUDA tensor")
        if table.dtype not in (torch.float32, torch.float64):
            raise ValueError("the table must be float32 or float64")
        table = table.contiguous()
        precision = 1 if table.dtype == torch.float64 else 0
        B = samples[0].n_anchors
        loss = torch.empty(B, dtype=table.dtype, device=table.device)
        stream = torch.cuda.current_stream(table.device).cuda_stream
        owner.ctx.ag_forward(samples, precision, table.data_ptr(), loss.data_ptr(), stream)
        ctx.owner, ctx.samples, ctx.precision = owner, samples, precision
        ctx.save_for_backward(table)
        return loss

    @staticmethod
    def backward(ctx, dloss):
        (table,) = ctx.saved_tensors
        dloss = dloss.contiguous().to(table.dtype)
        grad = torch.empty_like(table)
        stream = torch.cuda.current_stream(table.device).cuda_stream
        owner = ctx.owner
        # re-stage this batch (another call may have used the context since)
        owner.ctx.ag_forward(ctx.samples, ctx.precision, table.data_ptr(),
                             torch.empty_like(dloss).data_ptr(), stream)
        owner.ctx.ag_backward(dloss.data_ptr(), grad.data_ptr(), stream)
        return grad, None, None


class EPBatchLoss:
    """Differentiable EP batch loss bound to one graph and feature CSR."""

    def __init__(self, rows, cols, fptr, fids, n_feat: int, dims: int, loss: EPLoss,
                 grad_mode: str = "true", loss_weighting=None, device: int = 0):
        cfg = _native.default_config()
        cfg.dims, cfg.negatives = dims, loss.negatives
        cfg.loss, cfg.gamma, cfg.neg_margin = loss.code(), loss.gamma, loss.neg_margin
        cfg.grad_mode = _native.GRAD_TRUE if grad_mode == "true" else _native.GRAD_REFERENCE
        if loss_weighting is not None:
            cfg.loss_weighting, cfg.loss_weighting_exp = loss_weighting.kind, loss_weighting.weight
        cfg.device = device
        self.ctx = _native.Context(cfg)
        self.ctx.upload_graph(rows, cols, None)
        self.ctx.upload_features(fptr, fids, n_feat)
        self.n_feat, self.dims, self.negatives = n_feat, dims, loss.negatives

    def __call__(self, table: torch.Tensor, anchors, nbr_ptr, nbr, nbr_w, negatives) -> torch.Tensor:
        if tuple(table.shape) != (self.n_feat, self.dims):
            raise ValueError(f"table must have shape {(self.n_feat, self.dims)}")
        samples = _native.Context.samples(anchors, nbr_ptr, nbr, nbr_w, negatives)
        return _Fn.apply(table, self, samples)
