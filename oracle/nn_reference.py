"""CPU reference of the warm-start network (TEST INFRASTRUCTURE ONLY).

The same encoder-decoder as libps_b200.so's ps_nn_* entry points (4x4 pooling, x4 upsampling), in torch FP32 on the CPU, with
the GPU's bf16 roundings restated in the forward pass: the input, every weight and every hidden
activation are rounded to bf16 (round to nearest even), accumulation is FP32. The roundings pass
gradients straight through, so reference gradients are those of the FP32 computation on the
rounded values; the GPU additionally rounds each layer's pre-activation gradient to bf16 before
its GEMMs, hence the tolerances of the tests.

Parameters follow ps_nn_get_params: per layer W[cout][ky][kx][cin], then b[cout]; layers in the
order enc (2->c, c->c), (c->2c, 2c->2c), (2c->4c, 4c->4c), (4c->8c, 8c->8c), dec (12c->4c, 4c->4c),
(6c->2c, 2c->2c), (3c->c, c->c), out 1x1 (c->3), c = 32.
"""
from __future__ import annotations

import numpy as np


def layer_spec(c=32):
    return [(2, c, 3), (c, c, 3), (c, 2 * c, 3), (2 * c, 2 * c, 3), (2 * c, 4 * c, 3), (4 * c, 4 * c, 3),
            (4 * c, 8 * c, 3), (8 * c, 8 * c, 3), (12 * c, 4 * c, 3), (4 * c, 4 * c, 3), (6 * c, 2 * c, 3),
            (2 * c, 2 * c, 3), (3 * c, c, 3), (c, c, 3), (c, 3, 1)]


def unpack(params: np.ndarray, c=32):
    """-> list of (W [cout, cin, k, k] torch layout, b [cout]) as float32 numpy arrays."""
    out, o = [], 0
    for cin, cout, k in layer_spec(c):
        n = cout * k * k * cin
        W = params[o:o + n].reshape(cout, k, k, cin).transpose(0, 3, 1, 2).copy()
        o += n
        b = params[o:o + cout].copy()
        o += cout
        out.append((W, b))
    assert o == params.size
    return out


def pack(layers) -> np.ndarray:
    parts = []
    for W, b in layers:
        parts.append(np.asarray(W).transpose(0, 2, 3, 1).reshape(-1))
        parts.append(np.asarray(b).reshape(-1))
    return np.concatenate(parts).astype(np.float32)


class Reference:
    """forward(x [B,H,W,2] NHWC) -> y [B,H,W,3]; parameters as torch leaf tensors (grad enabled).

    round_grads=True also restates the GPU's backward roundings: the gradient entering each
    convolution (w.r.t. its output before the bias) is rounded to bf16, the bias gradient is
    not; the reference then differs from the GPU only by FP32 summation order."""

    def __init__(self, params: np.ndarray, c=32, round_grads=False):
        import torch

        self.torch = torch
        self.round_grads = round_grads
        self.layers = [(torch.tensor(W, requires_grad=True), torch.tensor(b, requires_grad=True))
                       for W, b in unpack(params, c)]

        class _RoundGrad(torch.autograd.Function):
            @staticmethod
            def forward(ctx, x):
                return x.view_as(x)

            @staticmethod
            def backward(ctx, g):
                return g.to(torch.bfloat16).to(torch.float32)

        self._round_grad = _RoundGrad.apply

        class _Forced(torch.autograd.Function):
            # value of a hidden activation taken from the GPU run; gradient masked by that value
            @staticmethod
            def forward(ctx, z, a):
                ctx.save_for_backward(a)
                return a.clone()

            @staticmethod
            def backward(ctx, g):
                (a,) = ctx.saved_tensors
                return g * (a > 0).to(g.dtype), None

        self._forced = _Forced.apply

    def _r(self, x):
        # bf16 round-to-nearest-even in the forward pass, identity gradient
        return x + (x.to(self.torch.bfloat16).to(self.torch.float32) - x).detach()

    def forward(self, x_nhwc, forced=None):
        """forced: optional list of the 14 hidden activations of a GPU run (NHWC); each hidden layer
        then outputs that value and masks its gradient with it, so that the backward pass sees the
        same activations and ReLU masks as the GPU's."""
        torch, F = self.torch, self.torch.nn.functional
        r = self._r
        x = r(torch.as_tensor(x_nhwc).permute(0, 3, 1, 2))

        def conv(i, a):
            W, b = self.layers[i]
            k = W.shape[-1]
            z = F.conv2d(a, r(W), None, padding=k // 2)
            if self.round_grads:
                z = self._round_grad(z)
            z = z + b.view(1, -1, 1, 1)
            if i < 14 and forced is not None:
                return self._forced(z, torch.as_tensor(forced[i]).permute(0, 3, 1, 2).contiguous())
            return r(F.relu(z)) if i < 14 else z

        def pool(a):
            return r(F.avg_pool2d(a, 4))

        def upcat(low, skip):
            return torch.cat([F.interpolate(low, scale_factor=4, mode="nearest"), skip], dim=1)

        a1 = conv(1, conv(0, x))
        a3 = conv(3, conv(2, pool(a1)))
        a5 = conv(5, conv(4, pool(a3)))
        a7 = conv(7, conv(6, pool(a5)))
        d2 = conv(9, conv(8, upcat(a7, a5)))
        d1 = conv(11, conv(10, upcat(d2, a3)))
        d0 = conv(13, conv(12, upcat(d1, a1)))
        y = conv(14, d0)
        return y.permute(0, 2, 3, 1)

    def grads(self) -> np.ndarray:
        return pack([(W.grad.detach().numpy(), b.grad.detach().numpy()) for W, b in self.layers])
