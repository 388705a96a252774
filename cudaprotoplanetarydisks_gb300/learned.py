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


# --------------------------------------------------------------------------
# the correction on a coarse disk, its training data and its training


def _fp(arr):
    return arr.ctypes.data_as(ctypes.POINTER(ctypes.c_float))


class Correction:
    """One trained network with its input normalisation (5 channel means, then 5
    deviations) and output scale.  step_DT advances a coarse disk one DT: the
    plain step, then the network's conservative density correction, applied only
    when the density stays positive and the mass change at roundoff."""

    def __init__(self, mlp, norm, scale):
        self.mlp = mlp
        self.norm = np.ascontiguousarray(norm, dtype=np.float32)
        self.scale = float(scale)
        self.lib = _capi.load()
        self.accepted = 0
        self.rejected = 0

    def features(self, disk, x):
        rc = self.lib.fargo_learned_features_ctx(disk.h, _fp(self.norm), ctypes.c_void_p(x.data_ptr()))
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_learned_features_ctx: status {rc}")

    def correction(self, x, y, ds, surf, nrad, nsec):
        """ds = divergence of the network's flux corrections for features x."""
        import torch
        self.mlp.forward(x, y)
        rc = self.lib.fargo_learned_divergence(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(surf.data_ptr()), nrad,
                                               nsec, ctypes.c_float(self.scale), ctypes.c_void_p(ds.data_ptr()), None)
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_learned_divergence: status {rc}")
        torch.cuda.synchronize()

    def step_DT(self, disk, work):
        """work: buffers from workspace(disk).  Returns (substeps, accepted)."""
        x, y, ds, surf = work
        self.features(disk, x)
        n = disk.step_DT()
        self.correction(x, y, ds, surf, disk.nrad, disk.nsec)
        acc = ctypes.c_int(0)
        dm = ctypes.c_double(0.0)
        rc = self.lib.fargo_learned_apply(disk.h, ctypes.c_void_p(ds.data_ptr()), ctypes.byref(acc), ctypes.byref(dm))
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_learned_apply: status {rc}")
        if acc.value:
            self.accepted += 1
        else:
            self.rejected += 1
        return n, bool(acc.value)


def workspace(disk):
    """Device buffers of one coarse disk: features, outputs, correction, surfaces."""
    import torch
    n = disk.nrad * disk.nsec
    surf = torch.tensor(disk.mesh()[3], dtype=torch.float64, device="cuda")
    return (torch.empty((n, NIN), dtype=torch.bfloat16, device="cuda"),
            torch.empty((n, NOUT), dtype=torch.float32, device="cuda"),
            torch.empty(n, dtype=torch.float32, device="cuda"), surf)


def fine_params(params, factor):
    """The fine teacher of a coarse disk: the same disk, factor x the cells in
    both directions."""
    fp = type(params)()
    ctypes.memmove(ctypes.byref(fp), ctypes.byref(params), ctypes.sizeof(params))
    fp.nrad, fp.nsec = params.nrad * factor, params.nsec * factor
    return fp


def density(disk, out):
    rc = _capi.load().fargo_learned_density(disk.h, ctypes.c_void_p(out.data_ptr()))
    if rc != _capi.FARGO_OK:
        raise RuntimeError(f"fargo_learned_density: status {rc}")


def restrict(fine, coarse, factor):
    rc = _capi.load().fargo_learned_restrict(fine.h, coarse.h, int(factor))
    if rc != _capi.FARGO_OK:
        raise RuntimeError(f"fargo_learned_restrict: status {rc}")


IDENTITY_NORM = np.array([0, 0, 0, 0, 0, 1, 1, 1, 1, 1], dtype=np.float32)


def generate(disks, factor=4, spinup=4, ndt=8, norm=None, precision=None):
    """Training pairs from the plain solver: for every (params, planets) of a
    coarse disk, its fine teacher runs `spinup` DTs, then for `ndt` DTs the
    coarse disk starts from the restricted fine state, takes one plain DT, and the
    target is the restricted fine density after the same DT minus the coarse one.
    Returns samples [(x, target, surf, nrad, nsec)] on the GPU."""
    import torch
    from . import Disk, FARGO_FP32_BULK
    prec = FARGO_FP32_BULK if precision is None else precision
    norm = IDENTITY_NORM if norm is None else norm
    samples = []
    for params, planets in disks:
        fine = Disk(fine_params(params, factor), planets, prec)
        coarse = Disk(params, planets, prec)
        fine.run(spinup)
        n = params.nrad * params.nsec
        surf = torch.tensor(coarse.mesh()[3], dtype=torch.float64, device="cuda")
        after = torch.empty(n, dtype=torch.float32, device="cuda")
        target_state = torch.empty(n, dtype=torch.float32, device="cuda")
        restrict(fine, coarse, factor)
        corr = Correction(None, norm, 1.0)
        for _ in range(ndt):
            x = torch.empty((n, NIN), dtype=torch.bfloat16, device="cuda")
            corr.features(coarse, x)
            coarse.step_DT()
            fine.step_DT()
            density(coarse, after)
            restrict(fine, coarse, factor)
            density(coarse, target_state)
            samples.append((x, (target_state - after).contiguous(), surf, params.nrad, params.nsec))
        fine.close()
        coarse.close()
    return samples


def feature_norm(samples, nsample=4):
    """Channel means and deviations of identity-normalised features."""
    import torch
    xs = torch.cat([s[0][:, :125].float().reshape(-1, 25, 5) for s in samples[:nsample]], dim=0)
    mean = xs.mean(dim=(0, 1))
    std = xs.std(dim=(0, 1)).clamp_min(1e-12)
    return np.concatenate([mean.cpu().numpy(), std.cpu().numpy()]).astype(np.float32)


def target_stats(samples):
    import torch
    t = torch.cat([s[1] for s in samples])
    return float(t.std()), float(t.var())


def _loss_call(lib, y, target, surf, nrad, nsec, scale, inv_var, buf):
    ds, e, dy, part, loss = buf
    rc = lib.fargo_learned_loss(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(target.data_ptr()),
                                ctypes.c_void_p(surf.data_ptr()), nrad, nsec, ctypes.c_float(scale),
                                ctypes.c_float(inv_var), ctypes.c_void_p(ds.data_ptr()), ctypes.c_void_p(e.data_ptr()),
                                ctypes.c_void_p(dy.data_ptr()), ctypes.c_void_p(part.data_ptr()),
                                ctypes.c_void_p(loss.data_ptr()), None)
    if rc != _capi.FARGO_OK:
        raise RuntimeError(f"fargo_learned_loss: status {rc}")


def _buffers(n):
    import torch
    return (torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"),
            torch.empty((n, NOUT), dtype=torch.float32, device="cuda"),
            torch.empty((n + 255) // 256, dtype=torch.float64, device="cuda"),
            torch.empty(1, dtype=torch.float64, device="cuda"))


def train(mlp, samples, scale, var, epochs=10, lr=2e-3, seed=0):
    """Adam on the normalised loss mean((ds - target)^2) / var over the samples,
    one sample (every cell of one coarse disk at one DT) per step.  Returns the
    loss of every step."""
    import torch
    lib = _capi.load()
    rng = np.random.default_rng(seed)
    n_max = max(s[3] * s[4] for s in samples)
    y = torch.empty((n_max, NOUT), dtype=torch.float32, device="cuda")
    buf = _buffers(n_max)
    losses = []
    for ep in range(epochs):
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / max(1, epochs)))
        for k in rng.permutation(len(samples)):
            x, target, surf, nrad, nsec = samples[k]
            n = nrad * nsec
            mlp.forward(x, y[:n], train=True)
            _loss_call(lib, y[:n], target, surf, nrad, nsec, scale, 1.0 / var, [b[:n] if b.dim() and b.shape[0] >= n
                                                                                   else b for b in buf])
            mlp.backward(x, buf[2][:n])
            mlp.adam(lr_ep)
            losses.append(float(buf[4].item()) / (n * var))
    torch.cuda.synchronize()
    return losses


def evaluate_loss(mlp, samples, scale, var):
    """Mean normalised loss of the network on samples, and of no correction."""
    import torch
    lib = _capi.load()
    n_max = max(s[3] * s[4] for s in samples)
    y = torch.empty((n_max, NOUT), dtype=torch.float32, device="cuda")
    buf = _buffers(n_max)
    with_net, without = [], []
    for x, target, surf, nrad, nsec in samples:
        n = nrad * nsec
        mlp.forward(x, y[:n])
        _loss_call(lib, y[:n], target, surf, nrad, nsec, scale, 1.0 / var, [b[:n] if b.dim() and b.shape[0] >= n
                                                                             else b for b in buf])
        with_net.append(float(buf[4].item()) / (n * var))
        without.append(float((target.double() ** 2).sum().item()) / (n * var))
    return float(np.mean(with_net)), float(np.mean(without))
