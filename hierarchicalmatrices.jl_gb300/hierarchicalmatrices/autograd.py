"""torch.autograd binding of the KernelMatrix product (the counterpart of a
ChainRulesCore rrule for the Julia API).

``kernel_matvec(H, w, x, y)`` returns H(x, y) w.  Its backward pass gives
    dL/dw = H^T g,   dL/dx = g .* (D_x w),   dL/dy = w .* (D_y^T g)
for the incoming gradient g, with the block tree of H held fixed (the tree is
a piecewise-constant function of the points).  ``x`` and ``y`` are the point
tensors H was built from; pass them with ``requires_grad`` to receive point
gradients.  All products run on the GPU (hm_mul, hm_mul_t, hm_mul_drow).
"""
import torch


class KernelMatvec(torch.autograd.Function):
    @staticmethod
    def forward(ctx, H, w, x, y):
        ctx.H = H
        ctx.save_for_backward(w)
        return H @ w.contiguous()

    @staticmethod
    def backward(ctx, g):
        (w,) = ctx.saved_tensors
        H = ctx.H
        g = g.contiguous()
        gw = gx = gy = None
        if ctx.needs_input_grad[1]:
            gw = H.T @ g
        if ctx.needs_input_grad[2]:
            d = torch.empty(H.shape[0], dtype=w.dtype, device=w.device)
            H.mul_drow(d, w.contiguous(), accumulate=False)
            gx = (g * d).to(ctx.saved_tensors[0].dtype)
        if ctx.needs_input_grad[3]:
            d = torch.empty(H.shape[1], dtype=w.dtype, device=w.device)
            H.mul_drow(d, g, transposed=True, accumulate=False)
            gy = w * d
        return None, gw, gx, gy


def kernel_matvec(H, w, x=None, y=None):
    """H(x, y) w with gradients for w and, when given, the points x and y."""
    if x is None:
        x = torch.zeros(0, device=w.device)
    if y is None:
        y = torch.zeros(0, device=w.device)
    return KernelMatvec.apply(H, w, x, y)
