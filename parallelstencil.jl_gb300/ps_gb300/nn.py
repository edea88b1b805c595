"""Learned warm start for the Stokes2D PT solver: a BF16 conv encoder-decoder whose convolutions
run as tcgen05 tensor-core GEMMs in libps_b200.so (no counterpart in the reference).

``gemm_bf16`` exposes the GEMM on its own (C = A B^T, bf16 operands, FP32 accumulation)."""
from __future__ import annotations

import ctypes

from . import _lib

RELU, OUT_BF16, ACCUMULATE = 1, 2, 4

_lib.register("ps_nn_gemm_bf16", [ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_int64, ctypes.c_int64,
                                  ctypes.c_int64, ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_void_p])


def gemm_bf16(A, B, C, bias=None, flags=0, split=1, stream=None):
    """C[M][N] (FP32, or bf16 with OUT_BF16) = A[M][K] @ B[N][K]^T (+ bias, ReLU) on the tensor cores.
    A, B, C, bias: contiguous CUDA tensors (torch)."""
    from .core import stream_handle

    M, K = A.shape
    N = B.shape[0]
    if B.shape[1] != K:
        raise ValueError("A and B must have the same K")
    _lib.call("ps_nn_gemm_bf16", ctypes.c_void_p(A.data_ptr()), ctypes.c_void_p(B.data_ptr()),
              ctypes.c_void_p(C.data_ptr()), M, N, K, ctypes.c_void_p(bias.data_ptr() if bias is not None else 0),
              int(flags), int(split), stream_handle(stream))


_V = ctypes.c_void_p
_lib.register("ps_nn_create", [ctypes.c_int64, ctypes.c_int64, ctypes.c_int32, ctypes.c_uint64, ctypes.POINTER(_V)])
_lib.register("ps_nn_destroy", [_V])
_lib.register("ps_nn_forward", [_V, _V, ctypes.c_int32, _V, _V])
_lib.register("ps_nn_backward", [_V, _V, _V])
_lib.register("ps_nn_zero_grad", [_V, _V])
_lib.register("ps_nn_adam_step", [_V, ctypes.c_float, ctypes.c_float, ctypes.c_float, ctypes.c_float, _V])
_lib.register("ps_nn_train_step", [_V, _V, _V, _V, ctypes.c_int32, ctypes.c_float, ctypes.POINTER(ctypes.c_double),
                                   _V])
_lib.register("ps_nn_get_activation", [_V, ctypes.c_int32, ctypes.POINTER(ctypes.c_float)])
_lib.register("ps_nn_param_count", [_V, ctypes.POINTER(ctypes.c_int64)])
_lib.register("ps_nn_get_params", [_V, ctypes.POINTER(ctypes.c_float)])
_lib.register("ps_nn_set_params", [_V, ctypes.POINTER(ctypes.c_float)])
_lib.register("ps_nn_get_grads", [_V, ctypes.POINTER(ctypes.c_float)])
_lib.register("ps_nn_set_scales", [_V, ctypes.POINTER(ctypes.c_float)])
_lib.register("ps_nn_get_scales", [_V, ctypes.POINTER(ctypes.c_float)])
_lib.register("ps_nn_save", [_V, ctypes.c_char_p])
_lib.register("ps_nn_load", [_V, ctypes.c_char_p])


def _p(t):
    return _V(t.data_ptr()) if t is not None else _V(0)


class Net:
    """The warm-start encoder-decoder held by the library (weights, Adam state, activations for
    batches up to ``max_batch`` of ``H x W`` images). Inputs / outputs are CUDA float32 tensors in
    NHWC layout: x [B, H, W, 2], y [B, H, W, 3]."""

    def __init__(self, H=256, W=256, max_batch=8, seed=1):
        from .core import require_initialized

        require_initialized()
        self.H, self.W, self.max_batch = H, W, max_batch
        h = _V()
        _lib.call("ps_nn_create", int(H), int(W), int(max_batch), int(seed), ctypes.byref(h))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            _lib.call("ps_nn_destroy", self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def forward(self, x, y=None, stream=None):
        import torch

        from .core import stream_handle

        B = x.shape[0]
        if y is None:
            y = torch.empty(B, self.H, self.W, 3, device=x.device, dtype=torch.float32)
        _lib.call("ps_nn_forward", self._h, _p(x.contiguous()), int(B), _p(y), stream_handle(stream))
        return y

    def backward(self, dy, stream=None):
        from .core import stream_handle

        _lib.call("ps_nn_backward", self._h, _p(dy.contiguous()), stream_handle(stream))

    def zero_grad(self, stream=None):
        from .core import stream_handle

        _lib.call("ps_nn_zero_grad", self._h, stream_handle(stream))

    def adam_step(self, lr, beta1=0.9, beta2=0.999, eps=1e-8, stream=None):
        from .core import stream_handle

        _lib.call("ps_nn_adam_step", self._h, float(lr), float(beta1), float(beta2), float(eps), stream_handle(stream))

    def train_step(self, x, t, lr, w=None, stream=None):
        from .core import stream_handle

        loss = ctypes.c_double()
        _lib.call("ps_nn_train_step", self._h, _p(x.contiguous()), _p(t.contiguous()),
                  _p(w.contiguous() if w is not None else None), int(x.shape[0]), float(lr), ctypes.byref(loss),
                  stream_handle(stream))
        return loss.value

    def param_count(self):
        n = ctypes.c_int64()
        _lib.call("ps_nn_param_count", self._h, ctypes.byref(n))
        return n.value

    def _host(self, name):
        import numpy as np

        a = np.empty(self.param_count(), dtype=np.float32)
        _lib.call(name, self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return a

    def activation(self, layer, B):
        """Output of layer `layer` (0..14) of the last forward pass of a batch of B, NHWC numpy."""
        import numpy as np

        lev = (0, 0, 1, 1, 2, 2, 3, 3, 2, 2, 1, 1, 0, 0, 0)[layer]
        c = (32, 32, 64, 64, 128, 128, 256, 256, 128, 128, 64, 64, 32, 32, 3)[layer]
        a = np.empty((B, self.H // 4 ** lev, self.W // 4 ** lev, c), dtype=np.float32)
        _lib.call("ps_nn_get_activation", self._h, int(layer), a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))
        return a

    def get_params(self):
        return self._host("ps_nn_get_params")

    def get_grads(self):
        return self._host("ps_nn_get_grads")

    def set_params(self, a):
        import numpy as np

        a = np.ascontiguousarray(a, dtype=np.float32)
        if a.size != self.param_count():
            raise ValueError("parameter vector of the wrong length")
        _lib.call("ps_nn_set_params", self._h, a.ctypes.data_as(ctypes.POINTER(ctypes.c_float)))

    @property
    def scales(self):
        s = (ctypes.c_float * 8)()
        _lib.call("ps_nn_get_scales", self._h, s)
        return list(s)

    @scales.setter
    def scales(self, v):
        s = (ctypes.c_float * 8)(*[float(x) for x in v])
        _lib.call("ps_nn_set_scales", self._h, s)

    def save(self, path):
        _lib.call("ps_nn_save", self._h, str(path).encode())

    def load(self, path):
        _lib.call("ps_nn_load", self._h, str(path).encode())


_lib.register("ps_stokes2d_warm_start", [_V, _V, ctypes.c_int32, _V])


def warm_start(net: Net, stokes, nvalid=255, stream=None):
    """Set stokes' Pt, Vx, Vy to the network's prediction for its Mus / Rog (FP64 fields)."""
    from .core import stream_handle

    _lib.call("ps_stokes2d_warm_start", net._h, ctypes.byref(stokes._fields), int(nvalid), stream_handle(stream))
