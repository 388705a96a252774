"""The learned coarse-grid correction: the stencil MLP (csrc/fargo_mlp.cu) behind
its C-ABI, on device buffers held by torch tensors.

The network maps a coarse cell's 5x5 neighbourhood of 5 channels (padded to 128
inputs) through two GELU layers of width 64 to 2 outputs, the radial and azimuthal
mass-flux corrections of the cell.  Weights and activations are BF16 on the tensor
cores with FP32 accumulation; the master weights and the optimiser (Adam) are
FP32.  Everything here launches the library's kernels; nothing is computed on the
host but the learning-rate schedule.
"""
import ctypes
import math

import numpy as np

from . import _capi

NIN, NH, NOUT, NOUTP = 128, 64, 2, 8
OFF_W1 = 0
OFF_B1 = OFF_W1 + NIN * NH
OFF_W2 = OFF_B1 + NH
OFF_B2 = OFF_W2 + NH * NH
OFF_W3 = OFF_B2 + NH
OFF_B3 = OFF_W3 + NH * NOUTP
NPARAM = OFF_B3 + NOUTP


def init_params(seed=0):
    """He-style initial weights (the output layer scaled down), zero biases; FP32."""
    rng = np.random.default_rng(seed)
    P = np.zeros(NPARAM, dtype=np.float32)
    P[OFF_W1:OFF_B1] = rng.normal(0.0, math.sqrt(2.0 / NIN), NIN * NH)
    P[OFF_W2:OFF_B2] = rng.normal(0.0, math.sqrt(2.0 / NH), NH * NH)
    w3 = np.zeros((NH, NOUTP), dtype=np.float32)
    w3[:, :NOUT] = rng.normal(0.0, 0.1 / math.sqrt(NH), (NH, NOUT))
    P[OFF_W3:OFF_B3] = w3.ravel()
    return P


class MLP:
    """fargo_mlp_*: forward/backward/Adam on at most max_rows rows per call.
    x: torch.bfloat16 [n, 128] on the GPU; y, dy: torch.float32 [n, 2]."""

    def __init__(self, max_rows, params=None, seed=0):
        self.lib = _capi.load()
        h = ctypes.c_void_p()
        rc = self.lib.fargo_mlp_create(int(max_rows), ctypes.byref(h))
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_mlp_create: status {rc}")
        self.h = h
        self.max_rows = int(max_rows)
        self.set_params(init_params(seed) if params is None else params)

    def _ok(self, rc, what):
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"{what}: status {rc}")

    def set_params(self, P):
        P = np.ascontiguousarray(P, dtype=np.float32)
        assert P.size == NPARAM
        self._ok(self.lib.fargo_mlp_set_params(self.h, P.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "set_params")

    def params(self):
        P = np.empty(NPARAM, dtype=np.float32)
        self._ok(self.lib.fargo_mlp_get_params(self.h, P.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "get_params")
        return P

    def grad(self):
        G = np.empty(NPARAM, dtype=np.float32)
        self._ok(self.lib.fargo_mlp_get_grad(self.h, G.ctypes.data_as(ctypes.POINTER(ctypes.c_float))), "get_grad")
        return G

    @staticmethod
    def _stream(stream):
        return ctypes.c_void_p(stream.cuda_stream) if stream is not None else None

    def forward(self, x, y, train=False, stream=None):
        n = x.shape[0]
        self._ok(self.lib.fargo_mlp_forward(self.h, ctypes.c_void_p(x.data_ptr()), n, ctypes.c_void_p(y.data_ptr()),
                                            1 if train else 0, self._stream(stream)), "forward")

    def backward(self, x, dy, stream=None):
        n = x.shape[0]
        self._ok(self.lib.fargo_mlp_backward(self.h, ctypes.c_void_p(x.data_ptr()), n, ctypes.c_void_p(dy.data_ptr()),
                                             self._stream(stream)), "backward")

    def adam(self, lr, stream=None):
        self._ok(self.lib.fargo_mlp_adam(self.h, ctypes.c_float(lr), self._stream(stream)), "adam")

    def close(self):
        if getattr(self, "h", None):
            self.lib.fargo_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass
