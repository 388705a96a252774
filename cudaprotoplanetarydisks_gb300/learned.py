"""The learned coarse-grid correction: the stencil MLP (csrc/fargo_mlp.cu) behind
its C-ABI, on device buffers held by torch tensors.

The network maps a coarse cell's 5x5 neighbourhood of 5 channels (padded to 128
inputs) through two GELU layers (tanh form) of width 64 to 2 outputs, the radial
and azimuthal mass-flux corrections of the cell.  Weights and activations are BF16 on the tensor
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
    x: torch.bfloat16 [n, 128] on the GPU; y, dy: torch.float32 [n, 2].  The
    backward pass recomputes the forward pass of its rows (train is ignored)."""

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

    def set_tensor_path(self, path):
        """"mma.sync" (default) or "tcgen05": the forward pass's tensor-core kernel."""
        code = {"tcgen05": 0, "mma.sync": 1}[path]
        self._ok(self.lib.fargo_mlp_set_tensor_path(self.h, code), "set_tensor_path")

    def status(self):
        """Raises if an MMA of a tcgen05 forward pass did not complete in time."""
        self._ok(self.lib.fargo_mlp_status(self.h), "mlp status")

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
    """One trained network with its input normalisation (125 means, then 125
    deviations) and output scale.  step_DT advances a coarse disk one DT: the
    plain step, then the network's conservative density correction, applied only
    when the density stays positive and the mass change at roundoff.
    ring_neutral: the radial outputs lose their ring means (fargo_learned_ring_center),
    so that the correction keeps every ring's mass (the averaged profile).
    limiter: beta of fargo_learned_divergence_limited (no cell gives more than that
    fraction of its mass), or None for the plain divergence."""

    def __init__(self, mlp, norm, scale, ring_neutral=False, limiter=None):
        self.mlp = mlp
        self.norm = np.ascontiguousarray(norm, dtype=np.float32)
        self.scale = float(scale)
        self.ring_neutral = bool(ring_neutral)
        self.limiter = limiter
        self.lib = _capi.load()
        self.accepted = 0
        self.rejected = 0
        self.rejected_mass = 0
        self.rejected_positivity = 0

    def features(self, disk, x):
        rc = self.lib.fargo_learned_features_ctx(disk.h, _fp(self.norm), ctypes.c_void_p(x.data_ptr()))
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_learned_features_ctx: status {rc}")

    def correction(self, x, y, ds, surf, nrad, nsec, disk=None):
        """ds = divergence of the network's flux corrections for features x (with
        the limiter on the grid and density of disk, when set)."""
        import torch
        self.mlp.forward(x, y)
        if self.ring_neutral:
            ring_center(y, nrad, nsec)
        if self.limiter is not None and disk is not None:
            # the limiter runs on the disk's own stream, which does not wait for
            # the default stream the network ran on
            torch.cuda.synchronize()
            rc = self.lib.fargo_learned_divergence_limited(disk.h, ctypes.c_void_p(y.data_ptr()),
                                                           ctypes.c_float(self.scale), ctypes.c_float(self.limiter),
                                                           ctypes.c_void_p(ds.data_ptr()))
            if rc != _capi.FARGO_OK:
                raise RuntimeError(f"fargo_learned_divergence_limited: status {rc}")
            return
        rc = self.lib.fargo_learned_divergence(ctypes.c_void_p(y.data_ptr()), ctypes.c_void_p(surf.data_ptr()), nrad,
                                               nsec, ctypes.c_float(self.scale), ctypes.c_void_p(ds.data_ptr()), None)
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_learned_divergence: status {rc}")
        torch.cuda.synchronize()

    def step_DT(self, disk, work):
        """work: buffers from workspace(disk).  Returns (substeps, accepted).  The
        network reads the plain step's result: over one DT the orbital advection
        carries the gas tens of cells in azimuth, so the correction is a function
        of the state it corrects, not of the state a DT earlier."""
        x, y, ds, surf = work
        n = disk.step_DT()
        self.features(disk, x)
        self.correction(x, y, ds, surf, disk.nrad, disk.nsec, disk)
        acc = ctypes.c_int(0)
        dm = ctypes.c_double(0.0)
        rc = self.lib.fargo_learned_apply(disk.h, ctypes.c_void_p(ds.data_ptr()), ctypes.byref(acc), ctypes.byref(dm))
        if rc != _capi.FARGO_OK:
            raise RuntimeError(f"fargo_learned_apply: status {rc}")
        if acc.value:
            self.accepted += 1
        else:
            self.rejected += 1
            # which judgement failed: the mass change against the correction's size
            # (the same test as the library's), else positivity or finiteness
            size = float((ds[:disk.nrad * disk.nsec].double().view(disk.nrad, disk.nsec).abs()
                          * surf[:disk.nrad].view(-1, 1)).sum())
            if abs(dm.value) > 1e-5 * size + 1e-300:
                self.rejected_mass += 1
            else:
                self.rejected_positivity += 1
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


IDENTITY_NORM = np.concatenate([np.zeros(125), np.ones(125)]).astype(np.float32)


def generate(disks, factor=4, spinup=4, ndt=8, norm=None, precision=None, reset_every=1, sample_every=1):
    """Training pairs from the plain solver: for every (params, planets) of a
    coarse disk, its fine teacher runs `spinup` DTs, then the coarse disk starts
    from the restricted fine state and both take `ndt` DTs; after each, the inputs
    are the coarse result and the target is the restricted fine density minus the
    coarse one.  The coarse disk restarts from the restricted fine state every
    `reset_every` DTs: with 1 every pair starts on the teacher's trajectory, with
    more the later pairs start from states the coarse solver drifted to, and their
    targets pull back to the teacher.  With sample_every = s > 1 the pairs spread
    along the teacher's trajectory: the teacher runs s - 1 DTs alone between two
    pairs, and every pair starts from the restricted teacher state.  Returns samples
    [(x, target, surf, nrad, nsec)] on the GPU."""
    import torch
    from . import Disk, FARGO_FP32_BULK
    prec = FARGO_FP32_BULK if precision is None else precision
    norm = IDENTITY_NORM if norm is None else norm
    samples = []
    for params, planets in disks:
        fine = Disk(fine_params(params, factor), planets, prec)
        coarse, ref = Disk(params, planets, prec), Disk(params, planets, prec)
        fine.run(spinup)
        n = params.nrad * params.nsec
        surf = torch.tensor(coarse.mesh()[3], dtype=torch.float64, device="cuda")
        after = torch.empty(n, dtype=torch.float32, device="cuda")
        target_state = torch.empty(n, dtype=torch.float32, device="cuda")
        restrict(fine, coarse, factor)
        corr = Correction(None, norm, 1.0)
        for k in range(ndt):
            if sample_every > 1:
                fine.run(sample_every - 1)
                restrict(fine, coarse, factor)
            x = torch.empty((n, NIN), dtype=torch.bfloat16, device="cuda")
            coarse.step_DT()
            fine.step_DT()
            corr.features(coarse, x)
            density(coarse, after)
            restrict(fine, ref, factor)
            density(ref, target_state)
            samples.append((x, (target_state - after).contiguous(), surf, params.nrad, params.nsec))
            if (k + 1) % reset_every == 0:
                restrict(fine, coarse, factor)
        for d in (fine, coarse, ref):
            d.close()
    return samples


def feature_norm(samples, nsample=8):
    """Means and deviations of each of the 125 identity-normalised inputs."""
    import torch
    xs = torch.cat([s[0][:, :125].float() for s in samples[:nsample]], dim=0)
    mean = xs.mean(dim=0)
    std = xs.std(dim=0).clamp_min(1e-12)
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


def ring_center(y, nrad, nsec):
    """fargo_learned_ring_center on the first nrad * nsec rows of y (in place)."""
    rc = _capi.load().fargo_learned_ring_center(ctypes.c_void_p(y.data_ptr()), nrad, nsec, None)
    if rc != _capi.FARGO_OK:
        raise RuntimeError(f"fargo_learned_ring_center: status {rc}")


def _buffers(n):
    import torch
    return (torch.empty(n, dtype=torch.float32, device="cuda"), torch.empty(n, dtype=torch.float32, device="cuda"),
            torch.empty((n, NOUT), dtype=torch.float32, device="cuda"),
            torch.empty((n + 255) // 256, dtype=torch.float64, device="cuda"),
            torch.empty(1, dtype=torch.float64, device="cuda"))


def _sample_var(target):
    return max(float((target.double() ** 2).mean().item()), 1e-300)


def train(mlp, samples, scale, var=None, epochs=10, lr=2e-3, seed=0, ring_neutral=False):
    """Adam on the loss mean((ds - target)^2) / mean(target^2) of one sample (every
    cell of one coarse disk at one DT) per step: each sample weighs the same
    whatever the size of its disk's correction (var: unused, kept for the
    signature).  ring_neutral: through the ring-mean projection of the radial
    outputs (its adjoint is itself).  Returns the mean loss of every epoch."""
    import torch
    lib = _capi.load()
    rng = np.random.default_rng(seed)
    n_max = max(s[3] * s[4] for s in samples)
    y = torch.empty((n_max, NOUT), dtype=torch.float32, device="cuda")
    buf = _buffers(n_max)
    norms = [_sample_var(s[1]) for s in samples]
    epoch_losses = []
    for ep in range(epochs):
        lr_ep = lr * 0.5 * (1.0 + math.cos(math.pi * ep / max(1, epochs)))
        acc = []
        for k in rng.permutation(len(samples)):
            x, target, surf, nrad, nsec = samples[k]
            n = nrad * nsec
            mlp.forward(x, y[:n], train=True)
            if ring_neutral:
                ring_center(y, nrad, nsec)
            _loss_call(lib, y[:n], target, surf, nrad, nsec, scale, 1.0 / norms[k],
                       [b[:n] if b.dim() and b.shape[0] >= n else b for b in buf])
            if ring_neutral:
                ring_center(buf[2], nrad, nsec)
            mlp.backward(x, buf[2][:n])
            mlp.adam(lr_ep)
            acc.append(float(buf[4].item()) / (n * norms[k]))
        epoch_losses.append(float(np.mean(acc)))
    torch.cuda.synchronize()
    return epoch_losses


def evaluate_loss(mlp, samples, scale, var=None, ring_neutral=False):
    """Mean over samples of mean((ds - target)^2) / mean(target^2) with the
    network's correction ds; without a correction that ratio is 1."""
    import torch
    lib = _capi.load()
    n_max = max(s[3] * s[4] for s in samples)
    y = torch.empty((n_max, NOUT), dtype=torch.float32, device="cuda")
    buf = _buffers(n_max)
    with_net = []
    for x, target, surf, nrad, nsec in samples:
        n = nrad * nsec
        v = _sample_var(target)
        mlp.forward(x, y[:n])
        if ring_neutral:
            ring_center(y, nrad, nsec)
        _loss_call(lib, y[:n], target, surf, nrad, nsec, scale, 1.0 / v,
                   [b[:n] if b.dim() and b.shape[0] >= n else b for b in buf])
        with_net.append(float(buf[4].item()) / (n * v))
    return float(np.mean(with_net)), 1.0


def experiment(n_train=12, n_test=4, nrad=256, factor=4, spinup=8, ndt_train=8, ndt_eval=10, epochs=40, lr=1e-3,
               seed=2025, sigma_noise=1e-4, reset_every=4, ring_neutral=True, limiter=0.5, sample_every=1,
               eval_every=1, ndt_time=10):
    """Coarse disks of nrad x 3 nrad drawn from the ensemble distribution, a
    factor-x finer plain run of each as teacher: train on n_train disks, then on
    n_test held-out disks report the one-DT loss with and without the network and
    a rollout of ndt_eval DTs from the restricted teacher state: after every DT
    the relative L2 error of the plain and the learned coarse density against the
    restricted teacher, at the end the same for the azimuthally averaged profile,
    then the wall time per DT of each run."""
    import time
    import torch
    from . import Disk, FARGO_FP32_BULK, c4_disks
    tr_disks = c4_disks(n_train, seed=seed, nrad_choices=(nrad,), sigma_noise=sigma_noise)
    te_disks = c4_disks(n_test, seed=seed + 1, nrad_choices=(nrad,), sigma_noise=sigma_noise)
    t0 = time.perf_counter()
    norm = feature_norm(generate(tr_disks[:2], factor, spinup, 2))
    tr = generate(tr_disks, factor, spinup, ndt_train, norm, reset_every=reset_every, sample_every=sample_every)
    ho = generate(te_disks, factor, spinup, 4, norm)
    t_gen = time.perf_counter() - t0
    scale, var = target_stats(tr)
    mlp = MLP(nrad * 3 * nrad, seed=seed)
    t0 = time.perf_counter()
    losses = train(mlp, tr, scale, var, epochs=epochs, lr=lr, ring_neutral=ring_neutral)
    t_train = time.perf_counter() - t0
    with_net, without = evaluate_loss(mlp, ho, scale, var, ring_neutral=ring_neutral)
    del tr, ho
    torch.cuda.empty_cache()
    corr = Correction(mlp, norm, scale, ring_neutral=ring_neutral, limiter=limiter)
    roll = []
    rel = lambda a, b: float(np.linalg.norm(a - b) / np.linalg.norm(b))  # noqa: E731
    for params, planets in te_disks:
        fine = Disk(fine_params(params, factor), planets, FARGO_FP32_BULK)
        fine.run(spinup)
        plain, learn, ref = (Disk(params, planets, FARGO_FP32_BULK) for _ in range(3))
        for d in (plain, learn, ref):
            restrict(fine, d, factor)
        work = workspace(learn)
        err = {"plain": [], "learned": []}
        perr = {"plain": [], "learned": []}
        for k in range(ndt_eval):
            fine.step_DT()
            plain.step_DT()
            corr.step_DT(learn, work)
            if (k + 1) % eval_every == 0:
                restrict(fine, ref, factor)
                r = ref.field("dens")[:-1]
                rp = r.mean(axis=1)
                for name, d in (("plain", plain), ("learned", learn)):
                    x = d.field("dens")[:-1]
                    err[name].append(rel(x, r))
                    perr[name].append(rel(x.mean(axis=1), rp))
        restrict(fine, ref, factor)
        prof = {k: d.field("dens")[:-1].mean(axis=1) for k, d in (("ref", ref), ("plain", plain), ("learned", learn))}
        t = {}
        for name, run in (("fine", lambda: fine.run(ndt_time)), ("plain", lambda: plain.run(ndt_time)),
                          ("learned", lambda: [corr.step_DT(learn, work) for _ in range(ndt_time)])):
            t0 = time.perf_counter()
            run()
            t[name] = (time.perf_counter() - t0) / ndt_time
        roll.append({"field_err": err, "profile_err": {k: rel(prof[k], prof["ref"]) for k in ("plain", "learned")},
                     "profile_err_per_eval": perr, "s_per_dt": t})
        for d in (fine, plain, learn, ref):
            d.close()
    avg = lambda get: float(np.mean([get(r) for r in roll]))  # noqa: E731
    return {
        "workload": f"{n_train} training and {n_test} held-out disks of the ensemble distribution at "
                    f"{nrad}x{3 * nrad}, teacher {factor * nrad}x{3 * factor * nrad} (plain method, FP32-bulk)",
        "ring_neutral": bool(ring_neutral),
        "limiter": limiter,
        "train": {"samples": n_train * ndt_train, "epochs": epochs, "first_epoch_loss": losses[0],
                  "last_epoch_loss": losses[-1],
                  "seconds_data": t_gen, "seconds_training": t_train},
        "held_out_one_dt_loss": {"with_network": with_net, "without": without},
        "rollout_dts": ndt_eval,
        "eval_every_dts": eval_every,
        "field_err_rel_per_dt": {k: [avg(lambda r, i=i, k=k: r["field_err"][k][i]) for i in range(ndt_eval // eval_every)]
                                 for k in ("plain", "learned")},
        "profile_err_rel_per_eval": {k: [avg(lambda r, i=i, k=k: r["profile_err_per_eval"][k][i])
                                         for i in range(ndt_eval // eval_every)] for k in ("plain", "learned")},
        "profile_err_rel_max_over_disks": {k: float(max(r["profile_err"][k] for r in roll))
                                           for k in ("plain", "learned")},
        "profile_err_rel": {k: avg(lambda r, k=k: r["profile_err"][k]) for k in ("plain", "learned")},
        "s_per_dt": {k: avg(lambda r, k=k: r["s_per_dt"][k]) for k in ("fine", "plain", "learned")},
        "corrections": {"accepted": corr.accepted, "rejected": corr.rejected,
                        "rejected_mass": corr.rejected_mass, "rejected_positivity": corr.rejected_positivity},
    }


def kernel_timing(nrad=256, reps=50, seed=5):
    """The correction's kernels on one nrad x 3 nrad disk: MLP forward and backward
    (with its gradient reduction) on the disk's rows of random inputs, timed with
    CUDA events over reps launches, and the features of the disk's state (a
    synchronous call: wall time).  Algorithmic flops per row: forward
    2 (128 64 + 64 64 + 64 2); backward the forward's layers 1-2 (recomputed), the
    data gradients dh2, dh1 and the weight gradients dW1, dW2, dW3."""
    import time
    import torch
    from . import Disk, FARGO_FP32_BULK, c4_disks
    (params, planets), = c4_disks(1, seed=seed, nrad_choices=(nrad,))
    disk = Disk(params, planets, FARGO_FP32_BULK)
    n = disk.nrad * disk.nsec
    mlp = MLP(n, seed=1)
    g = torch.Generator(device="cuda").manual_seed(seed)
    x = torch.randn((n, NIN), device="cuda", generator=g).to(torch.bfloat16)
    y = torch.empty((n, NOUT), device="cuda")
    dy = torch.randn((n, NOUT), device="cuda", generator=g)

    def ev(fn):
        fn()
        torch.cuda.synchronize()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record()
        for _ in range(reps):
            fn()
        b.record()
        torch.cuda.synchronize()
        return a.elapsed_time(b) / reps * 1e3

    mlp.set_tensor_path("tcgen05")
    fwd_tc_us = ev(lambda: mlp.forward(x, y))
    mlp.status()
    mlp.set_tensor_path("mma.sync")
    fwd_us, bwd_us = ev(lambda: mlp.forward(x, y)), ev(lambda: mlp.backward(x, dy))
    corr = Correction(mlp, IDENTITY_NORM, 1.0)
    corr.features(disk, x)
    t0 = time.perf_counter()
    for _ in range(reps):
        corr.features(disk, x)
    feat_us = (time.perf_counter() - t0) / reps * 1e6
    mlp.close()
    disk.close()
    f_fwd = 2 * (128 * 64 + 64 * 64 + 64 * 2)
    f_bwd = 2 * (128 * 64 + 64 * 64) + 2 * (2 * 64 + 64 * 64) + 2 * (128 * 64 + 64 * 64 + 64 * 2)
    return {"rows": n,
            "forward_path": "mma.sync m16n8k16 BF16, FP32 accumulate (default)",
            "forward_us": fwd_us, "forward_tflops": f_fwd * n / fwd_us * 1e-6,
            "forward_tcgen05_us": fwd_tc_us, "forward_tcgen05_tflops": f_fwd * n / fwd_tc_us * 1e-6,
            "forward_tcgen05_path": "tcgen05.mma kind::f16, FP32 accumulators in tensor memory, 128-row tiles",
            "x_bytes_per_forward": n * NIN * 2, "forward_x_GBs": n * NIN * 2 / fwd_us * 1e-3,
            "backward_path": "mma.sync m16n8k16 BF16, FP32 accumulate",
            "backward_us": bwd_us, "backward_tflops": f_bwd * n / bwd_us * 1e-6,
            "backward_includes": "forward recompute and the per-CTA gradient reduction",
            "features_wall_us": feat_us}


if __name__ == "__main__":
    import json
    import sys
    print(json.dumps(kernel_timing() if "--kernels" in sys.argv[1:] else experiment()))
