"""Learned Gauss-Newton warm start (no counterpart in the reference, which
starts every absolute reconstruction from the homogeneous distribution,
src/solver/solver.cpp:196-225).

A multilayer perceptron maps a frame's measured voltages, taken relative to
the voltages of the homogeneous distribution, to the parameter vector gamma
of every element.  Its training pairs are made by the forward solver itself
(EIT.solve on seeded inclusion phantoms), its training and inference run in
the library's own kernels (mpf_mlp_*: BF16 tcgen05 GEMMs with FP32
accumulation, Adam on FP32 master weights), and the plain Gauss-Newton
iteration decides: EIT.gn_solve_learned keeps a prediction only where it
lowers the data residual below the homogeneous start's and then iterates to
the target.
"""
from __future__ import annotations

import ctypes
import math
import time

import numpy as np

from ._ffi import check, lib, ptr


def _stream():
    import torch
    return ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)


def _f32(t, name: str):
    import torch
    if not (isinstance(t, torch.Tensor) and t.is_cuda and t.dtype == torch.float32):
        raise TypeError(f"{name} must be a float32 CUDA tensor")
    return t.contiguous()


class MLP:
    """in -> hidden1 -> hidden2 -> out perceptron with GELU hidden layers
    (mpf_mlp_create); widths are multiples of 128."""

    def __init__(self, inputs: int, hidden1: int, hidden2: int, outputs: int, seed: int = 0, device: int = 0):
        self.inputs, self.hidden1, self.hidden2, self.outputs = int(inputs), int(hidden1), int(hidden2), int(outputs)
        self.device = int(device)
        h = ctypes.c_void_p()
        check(lib().mpf_mlp_create(self.inputs, self.hidden1, self.hidden2, self.outputs, int(seed), self.device,
                                   ctypes.byref(h)))
        self._h = h
        off = np.zeros(7, np.int64)
        check(lib().mpf_mlp_layout(h, ptr(off)))
        self.offsets = off
        self.param_count = int(off[6])

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value:
            lib().mpf_mlp_destroy(h)
            self._h = None

    def forward(self, x):
        """y = net(x) for a (batch, inputs) float32 CUDA tensor."""
        import torch
        x = _f32(x, "x")
        y = torch.empty((x.shape[0], self.outputs), dtype=torch.float32, device=x.device)
        check(lib().mpf_mlp_forward(self._h, x.shape[0], ptr(x), ptr(y), self.outputs, _stream()))
        return y

    def backward(self, x, target, valid: int | None = None, want_loss: bool = True):
        """Gradients of the mean squared error over the first `valid` outputs;
        returns the loss (host sync) or None."""
        x = _f32(x, "x")
        target = _f32(target, "target")
        valid = int(valid if valid is not None else target.shape[1])
        loss = ctypes.c_double(0.0)
        check(lib().mpf_mlp_backward(self._h, x.shape[0], ptr(x), ptr(target), target.shape[1], valid,
                                     ctypes.byref(loss) if want_loss else None, _stream()))
        return loss.value if want_loss else None

    def adam(self, lr: float, beta1: float = 0.9, beta2: float = 0.999, eps: float = 1e-8,
             weight_decay: float = 0.0):
        """One Adam step from the last backward's gradients (mpf_mlp_adam);
        decoupled weight decay on the weight matrices."""
        check(lib().mpf_mlp_adam(self._h, float(lr), float(beta1), float(beta2), float(eps), float(weight_decay),
                                 _stream()))

    def train_step(self, x, target, rows=None, valid: int | None = None, lr: float = 1e-3, beta1: float = 0.9,
                   beta2: float = 0.999, eps: float = 1e-8, weight_decay: float = 0.0, want_loss: bool = False):
        """backward() + adam() on the batch rows `rows` (int32 CUDA tensor)
        of x and target without gathering them (mpf_mlp_train_step); rows
        None takes every row of x.  Returns the loss (host sync) or None."""
        import torch
        x = _f32(x, "x")
        target = _f32(target, "target")
        if rows is None:
            batch, rp = x.shape[0], None
        else:
            rows = rows.to(device=x.device, dtype=torch.int32).contiguous()
            batch, rp = rows.shape[0], ptr(rows)
        valid = int(valid if valid is not None else target.shape[1])
        loss = ctypes.c_double(0.0)
        check(lib().mpf_mlp_train_step(self._h, batch, ptr(x), x.shape[1], rp, ptr(target), target.shape[1], valid,
                                       float(lr), float(beta1), float(beta2), float(eps), float(weight_decay),
                                       ctypes.byref(loss) if want_loss else None, _stream()))
        return loss.value if want_loss else None

    def _params(self, which: int, buf=None):
        import torch
        if buf is None:
            buf = torch.empty(self.param_count, dtype=torch.float32, device=f"cuda:{self.device}")
        check(lib().mpf_mlp_params(self._h, ptr(buf), which, _stream()))
        return buf

    def parameters(self):
        """Flat FP32 parameters W1 | b1 | W2 | b2 | W3 | b3 (see offsets)."""
        return self._params(0)

    def set_parameters(self, buf):
        """Load a flat FP32 parameter vector (resets the Adam state)."""
        self._params(1, _f32(buf, "parameters"))

    def gradients(self):
        """Flat FP32 gradients of the last backward, laid out as parameters()."""
        return self._params(2)

    # checkpoint file: 8-byte magic, int64 inputs, hidden1, hidden2, outputs,
    # parameter count, then the FP32 master parameters (little-endian, the
    # layout of parameters()); the Adam state is not kept
    MAGIC = b"MPFMLP01"

    def save(self, path: str) -> None:
        """Write the trained parameters to a binary checkpoint."""
        flat = self.parameters().detach().cpu().numpy().astype("<f4")
        head = np.array([self.inputs, self.hidden1, self.hidden2, self.outputs, self.param_count], dtype="<i8")
        with open(path, "wb") as fh:
            fh.write(self.MAGIC)
            fh.write(head.tobytes())
            fh.write(flat.tobytes())

    @staticmethod
    def read_checkpoint(path: str):
        """(dims (inputs, hidden1, hidden2, outputs), FP32 parameters) of a
        checkpoint written by save(); ValueError for a file of another kind
        or of the wrong length."""
        with open(path, "rb") as fh:
            data = fh.read()
        if len(data) < 48 or data[:8] != MLP.MAGIC:
            raise ValueError(f"{path}: not a network checkpoint")
        head = np.frombuffer(data[8:48], dtype="<i8")
        count = int(head[4])
        if len(data) != 48 + 4 * count:
            raise ValueError(f"{path}: {len(data)} bytes, expected {48 + 4 * count} for {count} parameters")
        return tuple(int(v) for v in head[:4]), np.frombuffer(data[48:], dtype="<f4")

    @classmethod
    def load(cls, path: str, device: int = 0) -> "MLP":
        """A network with the dimensions and parameters of a checkpoint."""
        import torch
        dims, flat = cls.read_checkpoint(path)
        net = cls(*dims, seed=0, device=device)
        if flat.size != net.param_count:
            raise ValueError(f"{path}: {flat.size} parameters, the network has {net.param_count}")
        net.set_parameters(torch.tensor(flat, device=f"cuda:{device}"))
        return net

    def unpack(self, flat):
        """Split a flat parameter (or gradient) vector into (W1, b1, W2, b2, W3, b3) numpy arrays."""
        f = flat.detach().cpu().numpy() if hasattr(flat, "detach") else np.asarray(flat)
        o = self.offsets
        W1 = f[o[0]:o[0] + self.hidden1 * self.inputs].reshape(self.hidden1, self.inputs)
        b1 = f[o[1]:o[1] + self.hidden1]
        W2 = f[o[2]:o[2] + self.hidden2 * self.hidden1].reshape(self.hidden2, self.hidden1)
        b2 = f[o[3]:o[3] + self.hidden2]
        W3 = f[o[4]:o[4] + self.outputs * self.hidden2].reshape(self.outputs, self.hidden2)
        b3 = f[o[5]:o[5] + self.outputs]
        return W1, b1, W2, b2, W3, b3


def zero_network(inputs: int, outputs: int, device: int = 0) -> MLP:
    """A network whose output is exactly zero (last layer zero): with a
    linear prior set, mpf_gn_solve_learned then starts from the prior
    alone."""
    import torch
    net = MLP(inputs, 128, 128, outputs, seed=0, device=device)
    flat = net.parameters()
    flat[int(net.offsets[4]):].zero_()
    net.set_parameters(flat)
    return net


def round_up(v: int, m: int) -> int:
    """v rounded up to a multiple of m."""
    return (v + m - 1) // m * m


def inclusion_frames(centroids: np.ndarray, count: int, rng: np.random.Generator, inclusions=(1, 3),
                     radius=(0.05, 0.3), contrast=(0.1, 10.0), domain_radius: float = 1.0) -> np.ndarray:
    """Log-conductivity frames in the library's dB parametrisation
    (sigma = ref 10^(gamma/10)): a 0 dB background with 1-3 disks of radius
    U(radius) and conductivity ratio log-uniform in `contrast`, centres
    uniform in the disk that keeps the inclusion inside the domain."""
    E = centroids.shape[0]
    out = np.zeros((count, E), np.float32)
    lo, hi = np.log(contrast[0]), np.log(contrast[1])
    for f in range(count):
        k = rng.integers(inclusions[0], inclusions[1] + 1)
        for _ in range(k):
            r = rng.uniform(*radius)
            rc = (domain_radius - r) * math.sqrt(rng.uniform())
            th = rng.uniform(0.0, 2.0 * math.pi)
            c = np.array([rc * math.cos(th), rc * math.sin(th)])
            ratio = math.exp(rng.uniform(lo, hi))
            inside = ((centroids - c) ** 2).sum(axis=1) <= r * r
            out[f, inside] = 10.0 * math.log10(ratio)
    return out


def generate_pairs(model, gammas: np.ndarray, batch: int = 64, options=None):
    """Voltages of the forward model for every frame of `gammas` (count x E,
    host).  Returns (V as (count, Mm, Md), gamma) CUDA tensors."""
    import torch
    from .eit import SolveOptions
    opts = options or SolveOptions(tol=1e-5, max_iter=6000)
    Vs = []
    for i in range(0, gammas.shape[0], batch):
        g = torch.tensor(gammas[i:i + batch], device=f"cuda:{model.device}")
        Vs.append(model.solve(g, opts).contiguous())
    return torch.cat(Vs), torch.tensor(gammas, device=f"cuda:{model.device}")


def gn_labels(model, V, lam: float, target: float = 1e-3, max_iters: int = 4, batch: int = 64, options=None,
              net0=None):
    """Training targets of the learned start over the model's linear prior
    (EIT.learned_prior): for every frame of V (count, Mm, Md), where batched
    Gauss-Newton from the prior converges (relative data residual <=
    target).  A frame that does not get there within max_iters updates keeps
    the prior itself (zero correction).  Returns (labels (count x E) CUDA
    tensor, fraction of frames that converged).  `net0`: the network whose
    output is added to the prior during the GN runs, a zero network
    (`zero_network`) by default."""
    import torch
    if getattr(model, "prior_lambda", None) is None:
        raise ValueError("gn_labels needs the model's linear prior (EIT.learned_prior)")
    E = model.mesh.elements.shape[0]
    L = V.shape[1] * V.shape[2]
    if net0 is None:
        net0 = zero_network(L, round_up(E, 128), device=model.device)
    out = torch.empty((V.shape[0], E), dtype=torch.float32, device=V.device)
    converged = 0
    for i in range(0, V.shape[0], batch):
        Vb = V[i:i + batch].contiguous()
        g, _, res, _, _ = model.gn_solve_learned(net0, Vb, lam, target=target, max_iters=max_iters, options=options)
        bad = np.flatnonzero(~(res <= target))
        if bad.size:
            idx = torch.tensor(bad, device=V.device)
            g[idx] = model.learned_prior_apply(model.learned_input(Vb[idx].contiguous()))
        converged += Vb.shape[0] - bad.size
        out[i:i + Vb.shape[0]] = g
    return out, converged / V.shape[0]


def add_noise(V, snr_db: float, generator=None):
    """V + Gaussian noise with std rms(V_frame) 10^(-snr/20) per frame."""
    import torch
    rms = V.reshape(V.shape[0], -1).pow(2).mean(dim=1).sqrt()
    std = rms * 10.0 ** (-snr_db / 20.0)
    noise = torch.randn(V.shape, device=V.device, generator=generator) * std.view(-1, *([1] * (V.dim() - 1)))
    return V + noise


def train_warm_start(model, net: MLP, V, gamma, epochs: int = 60, batch: int = 256, lr: float = 1e-3,
                     weight_decay: float = 1e-4, snr_db: float | None = 60.0, seed: int = 0, log=None,
                     prior: bool = False):
    """Train `net` on (V, gamma) pairs with Adam and a cosine learning rate;
    fresh measurement noise at `snr_db` every epoch (None: noise-free).
    With `prior` the model's linear prior is set (EIT.learned_prior) and the
    network learns gamma - prior(x), the correction to the linear
    Gauss-Newton step, as mpf_gn_solve_learned then starts from
    prior(x) + net(x).  Returns the per-epoch mean losses and the wall time."""
    import torch
    N, E = gamma.shape
    if batch % 128:
        raise ValueError("batch must be a multiple of 128")
    gen = torch.Generator(device=V.device)
    gen.manual_seed(seed)
    steps_per_epoch = max(1, N // batch)
    total = epochs * steps_per_epoch
    if prior and getattr(model, "prior_lambda", None) is None:
        raise ValueError("prior=True needs the model's linear prior (EIT.learned_prior)")
    losses = []
    # the first use of the random-number and permutation kernels at these
    # sizes loads them (seconds on a fresh process): outside the timed loop,
    # with a generator of its own so the training draws are unchanged
    warm = torch.Generator(device=V.device)
    warm.manual_seed(seed + 1)
    if snr_db is not None:
        add_noise(V, snr_db, warm)
    torch.randperm(N, device=V.device, generator=warm)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    step = 0
    T = torch.empty_like(gamma) if prior else gamma
    for ep in range(epochs):
        Vn = add_noise(V, snr_db, gen) if snr_db is not None else V
        X = model.learned_input(Vn)
        if prior:
            T.copy_(gamma)
            model.learned_prior_apply(X, T, mode=-1)
        perm = torch.randperm(N, device=V.device, generator=gen).to(torch.int32)
        acc = 0.0
        for b in range(steps_per_epoch):
            idx = perm[b * batch:(b + 1) * batch]
            want = b == steps_per_epoch - 1
            cur = lr * 0.5 * (1.0 + math.cos(math.pi * step / total))
            loss = net.train_step(X, T, rows=idx, valid=E, lr=cur, weight_decay=weight_decay, want_loss=want)
            if want:
                acc = loss
            step += 1
        losses.append(acc)
        if log:
            log(f"epoch {ep}: loss {acc:.4g}")
    torch.cuda.synchronize()
    return losses, time.perf_counter() - t0
