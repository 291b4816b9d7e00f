"""The surrogate's MLP on the tensor cores (C ABI bldfm_surrogate_*).

8 input features -> four GELU hidden layers of 256 -> 4 outputs; the 256 x 256
layers run forward and backward as tcgen05 BF16 GEMMs with FP32 accumulation;
the last hidden layer and the output layer stay FP32; FP32 master weights
trained with Adam.  Tensors are torch CUDA tensors; loss weights are per
sample and output, shape (n, 4).
"""

import ctypes

import numpy as np
import torch

from . import _lib

N_IN, N_HIDDEN, N_OUT, X_STRIDE = 8, 256, 4, 8


class MLP:
    def __init__(self, batch=65536, seed=0):
        self.lib = _lib.load()
        self.batch = int(batch)
        h = ctypes.c_void_p()
        _lib.check(self.lib.bldfm_surrogate_create(self.batch, int(seed), ctypes.byref(h)), "surrogate_create")
        self.h = h
        self.nparams = int(self.lib.bldfm_surrogate_nparams())

    def close(self):
        if self.h:
            self.lib.bldfm_surrogate_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def params(self):
        p = np.empty(self.nparams, dtype=np.float32)
        _lib.check(self.lib.bldfm_surrogate_params(self.h, _lib.ptr(p), None), "surrogate_params")
        return p

    def set_params(self, p):
        p = np.ascontiguousarray(p, dtype=np.float32)
        assert p.size == self.nparams
        _lib.check(self.lib.bldfm_surrogate_params(self.h, None, _lib.ptr(p)), "surrogate_params")

    def grads(self):
        g = np.empty(self.nparams, dtype=np.float32)
        loss = np.zeros(1, dtype=np.float32)
        _lib.check(self.lib.bldfm_surrogate_grads(self.h, _lib.ptr(g), _lib.ptr(loss)), "surrogate_grads")
        return g, float(loss[0])

    def train_step(self, X, T, w, lr, stream=None):
        n = X.shape[0]
        s = (stream or torch.cuda.current_stream()).cuda_stream
        _lib.check(
            self.lib.bldfm_surrogate_train_step(
                self.h, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(T.data_ptr()), ctypes.c_void_p(w.data_ptr()),
                n, float(lr), ctypes.c_void_p(s),
            ),
            "surrogate_train_step",
        )

    def forward(self, X, Y=None, stream=None):
        n = X.shape[0]
        if Y is None:
            Y = torch.empty((n, N_OUT), dtype=torch.float32, device=X.device)
        s = (stream or torch.cuda.current_stream()).cuda_stream
        _lib.check(
            self.lib.bldfm_surrogate_forward(self.h, ctypes.c_void_p(X.data_ptr()), ctypes.c_void_p(Y.data_ptr()), n,
                                             ctypes.c_void_p(s)),
            "surrogate_forward",
        )
        return Y


def param_slices():
    """Offsets of the parameter blocks in the flat vector."""
    H = N_HIDDEN
    out = {"W0": (0, N_IN * H), "b0": (N_IN * H, N_IN * H + H)}
    o = N_IN * H + H
    for j in (1, 2, 3):
        out["Wt%d" % j] = (o, o + H * H)
        out["b%d" % j] = (o + H * H, o + H * H + H)
        o += H * H + H
    out["W4"] = (o, o + H * N_OUT)
    out["b4"] = (o + H * N_OUT, o + H * N_OUT + N_OUT)
    return out
