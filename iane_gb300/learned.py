"""Learned warm start for 3-D Richardson-Lucy: a small encoder-decoder CNN.

Architecture (3 levels, 16/32/64 channels, 3x3x3 convolutions, ReLU, average pooling,
nearest upsampling, skip connections by channel concatenation, residual head):

    input  [2]: observed / mean(observed), PSF sigma / 3 (constant channel)
    e1a 2->16, e1b 16->16 | pool | e2a 16->32, e2b 32->32 | pool | e3a 32->64, e3b 64->64,
    e3c 64->64 | up | d2a (64+32)->32, d2b 32->32 | up | d1a (32+16)->16, d1b 16->16 | head 16->1
    output = observed / mean + head  (times the mean: the RL start, floored at eps)

464,785 parameters (about 0.46 M). Activations and weights are BF16, accumulation FP32, master weights
FP32 with Adam. Every operation runs in libiane_gb300.so (iane_gb_cnn_*); torch supplies
device memory only. Training pairs are generated here: ellipsoid phantoms blurred by random
Gaussian PSFs with Poisson noise, paired with long FP32 Richardson-Lucy runs of this library.
"""
from __future__ import annotations

import ctypes
import struct
from pathlib import Path

import numpy as np

from . import RichardsonLucy, convolve
from ._lib import check, lib

LAYERS = [
    # name, input channels, output channels, relu
    ("e1a", 2, 16, True), ("e1b", 16, 16, True),
    ("e2a", 16, 32, True), ("e2b", 32, 32, True),
    ("e3a", 32, 64, True), ("e3b", 64, 64, True), ("e3c", 64, 64, True),
    ("d2a", 96, 32, True), ("d2b", 32, 32, True),
    ("d1a", 48, 16, True), ("d1b", 16, 16, True),
    ("head", 16, 1, False),
]
MAGIC = b"IANEGBWS"


def _p(t) -> int:
    return t.data_ptr() if t is not None else None


class WarmStartNet:
    def __init__(self, device="cuda", seed: int = 0, stream=None):
        import torch

        self.torch = torch
        self.device = torch.device(device)
        self.stream = stream
        self.offsets = {}
        n = 0
        for name, ci, co, _ in LAYERS:
            self.offsets[name] = (n, n + co * ci * 27)  # weights, then co biases
            n += co * ci * 27 + co
        self.size = n
        rng = np.random.default_rng(seed)
        host = np.zeros(n, np.float32)
        for name, ci, co, _ in LAYERS:
            w0, b0 = self.offsets[name]
            std = np.sqrt(2.0 / (ci * 27)) if name != "head" else 1e-3
            host[w0:b0] = rng.standard_normal(co * ci * 27).astype(np.float32) * np.float32(std)
        self.master = torch.from_numpy(host).to(self.device)
        self.p16 = self.master.to(torch.bfloat16)
        self.grad = torch.zeros_like(self.master)
        self.m = torch.zeros_like(self.master)
        self.v = torch.zeros_like(self.master)
        self.steps = 0
        self._flipped = None
        self._packed = None
        self._buffers = {}

    # -- parameter views ------------------------------------------------------------------
    def w16(self, name):
        w0, b0 = self.offsets[name]
        return self.p16[w0:b0]

    def bias(self, name):
        _, b0 = self.offsets[name]
        co = [l[2] for l in LAYERS if l[0] == name][0]
        return self.master[b0:b0 + co]

    def dw(self, name):
        w0, b0 = self.offsets[name]
        return self.grad[w0:b0]

    def db(self, name):
        _, b0 = self.offsets[name]
        co = [l[2] for l in LAYERS if l[0] == name][0]
        return self.grad[b0:b0 + co]

    def _stream(self):
        s = self.stream if self.stream is not None else self.torch.cuda.current_stream(self.device)
        return s.cuda_stream

    # -- buffers per volume shape -----------------------------------------------------------
    def _buf(self, shape):
        """Forward buffers for one volume shape: C8 activations (octets, D, H, W, 8), zeroed
        so that unused octet slots hold zeros, and the FP32 output and residual."""
        key = tuple(shape)
        if key in self._buffers:
            return self._buffers[key]
        torch = self.torch
        d, h, w = key
        if d % 4 or h % 4 or w % 4:
            raise ValueError("volume extents must be multiples of 4 (two 2x poolings)")
        s1, s2, s3 = (d, h, w), (d // 2, h // 2, w // 2), (d // 4, h // 4, w // 4)
        b = {"x16": self._act(2, s1)}
        for name, c, s in (("e1a", 16, s1), ("e1b", 16, s1), ("p1", 16, s2), ("e2a", 32, s2), ("e2b", 32, s2),
                           ("p2", 32, s3), ("e3a", 64, s3), ("e3b", 64, s3), ("e3c", 64, s3), ("u2", 64, s2),
                           ("d2a", 32, s2),
                           ("d2b", 32, s2), ("u1", 32, s1), ("d1a", 16, s1), ("d1b", 16, s1)):
            b[name] = self._act(c, s)
        b["out"] = torch.empty((1,) + s1, dtype=torch.float32, device=self.device)
        b["res"] = torch.empty((1,) + s1, dtype=torch.float32, device=self.device)
        b["loss"] = torch.zeros(1, dtype=torch.float64, device=self.device)
        self._buffers[key] = b
        return b

    def _act(self, c, s):
        return self.torch.zeros(((c + 7) // 8,) + tuple(s) + (8,), dtype=self.torch.bfloat16, device=self.device)

    def _grad_buf(self, shape):
        """Gradient buffers (allocated on the first backward of a shape)."""
        b = self._buf(shape)
        if "g_out" in b:
            return b
        d, h, w = shape
        s1, s2, s3 = (d, h, w), (d // 2, h // 2, w // 2), (d // 4, h // 4, w // 4)
        for name, c, s in (("g_out", 1, s1), ("g16a", 16, s1), ("g16b", 16, s1), ("g_cat1", 48, s1),
                           ("g32a", 32, s2), ("g32b", 32, s2), ("g_cat2", 96, s2), ("g64a", 64, s3),
                           ("g64b", 64, s3), ("g_p2", 32, s3), ("g_p1", 16, s2)):
            b[name] = self._act(c, s)
        need = 0
        for name, ci, co, _ in LAYERS:
            ls = {"e1": s1, "e2": s2, "e3": s3, "d2": s2, "d1": s1, "he": s1}[name[:2]]
            c0, c1 = {"d2a": (64, 32), "d1a": (32, 16)}.get(name, (ci, 0))
            need = max(need, lib().iane_gb_cnn_wgrad_scratch_bytes(c0, c1, *ls, co))
        b["wg"] = self.torch.empty(int(need) + 256, dtype=self.torch.uint8, device=self.device)
        return b

    # -- operations ---------------------------------------------------------------------------
    def _conv(self, x0, c0, x1, c1, shape, weights, bias, co, y16=None, y32=None, residual=None, relu=True,
              mask=None):
        check(lib().iane_gb_cnn_conv3(_p(x0), c0, _p(x1), c1, shape[0], shape[1], shape[2], _p(weights), _p(bias),
                                      co, _p(y16), _p(y32), _p(residual), 1 if relu else 0, _p(mask),
                                      self._stream()))

    def _wgrad(self, b, x0, c0, x1, c1, shape, dy, co, name):
        scratch = b["wg"]
        check(lib().iane_gb_cnn_conv3_wgrad(_p(x0), c0, _p(x1), c1, shape[0], shape[1], shape[2], _p(dy), co,
                                            _p(self.dw(name)), _p(self.db(name)), _p(scratch), scratch.numel(),
                                            self._stream()))

    def _flips(self):
        if self._flipped is None:
            torch = self.torch
            self._flipped = {}
            for name, ci, co, _ in LAYERS:
                out = torch.empty(ci * co * 27, dtype=torch.bfloat16, device=self.device)
                check(lib().iane_gb_cnn_flip(_p(self.w16(name)), co, ci, _p(out), self._stream()))
                self._flipped[name] = out
        return self._flipped

    def _packs(self):
        """Weights packed for the tensor-core forward (refreshed after each update)."""
        if self._packed is None:
            torch = self.torch
            self._packed = {}
            for name, ci, co, _ in LAYERS:
                c0, c1 = {"d2a": (64, 32), "d1a": (32, 16)}.get(name, (ci, 0))
                out = torch.empty(int(lib().iane_gb_cnn_tc_packed_bytes(co, c0, c1)) // 2, dtype=torch.bfloat16,
                                  device=self.device)
                check(lib().iane_gb_cnn_tc_pack(_p(self.w16(name)), co, c0, c1, _p(out), self._stream()))
                self._packed[name] = out
        return self._packed

    def forward(self, observed_norm, sigma: float, tensor_cores: bool = False):
        """observed_norm: f32 tensor (D, H, W) = observed / mean(observed). Returns the
        (1, D, H, W) f32 output (normalised estimate); activations stay for backward().
        tensor_cores=True runs every convolution on the tcgen05 kernel (inference); the
        default SIMT kernels are the ones the backward pass mirrors."""
        shape = tuple(observed_norm.shape)
        b = self._buf(shape)
        s1 = shape
        s2 = tuple(v // 2 for v in shape)
        s3 = tuple(v // 4 for v in shape)
        st = self._stream()
        b["res"][0].copy_(observed_norm)
        b["x16"][0, ..., 0].copy_(observed_norm)
        b["x16"][0, ..., 1].fill_(sigma / 3.0)
        packs = self._packs() if tensor_cores else None

        def c(name, x0, c0, x1, c1, s, co, y16=None, y32=None, residual=None, relu=True):
            if packs is not None:
                check(lib().iane_gb_cnn_conv3_tc(_p(x0), c0, _p(x1), c1, s[0], s[1], s[2], _p(packs[name]),
                                                 _p(self.bias(name)), co, _p(y16), _p(y32), _p(residual),
                                                 1 if relu else 0, st))
            else:
                self._conv(x0, c0, x1, c1, s, self.w16(name), self.bias(name), co, y16=y16, y32=y32,
                           residual=residual, relu=relu)

        c("e1a", b["x16"], 2, None, 0, s1, 16, y16=b["e1a"])
        c("e1b", b["e1a"], 16, None, 0, s1, 16, y16=b["e1b"])
        check(lib().iane_gb_cnn_pool2(_p(b["e1b"]), 16, *s1, _p(b["p1"]), st))
        c("e2a", b["p1"], 16, None, 0, s2, 32, y16=b["e2a"])
        c("e2b", b["e2a"], 32, None, 0, s2, 32, y16=b["e2b"])
        check(lib().iane_gb_cnn_pool2(_p(b["e2b"]), 32, *s2, _p(b["p2"]), st))
        c("e3a", b["p2"], 32, None, 0, s3, 64, y16=b["e3a"])
        c("e3b", b["e3a"], 64, None, 0, s3, 64, y16=b["e3b"])
        c("e3c", b["e3b"], 64, None, 0, s3, 64, y16=b["e3c"])
        check(lib().iane_gb_cnn_up2(_p(b["e3c"]), 64, *s3, _p(b["u2"]), st))
        c("d2a", b["u2"], 64, b["e2b"], 32, s2, 32, y16=b["d2a"])
        c("d2b", b["d2a"], 32, None, 0, s2, 32, y16=b["d2b"])
        check(lib().iane_gb_cnn_up2(_p(b["d2b"]), 32, *s2, _p(b["u1"]), st))
        c("d1a", b["u1"], 32, b["e1b"], 16, s1, 16, y16=b["d1a"])
        c("d1b", b["d1a"], 16, None, 0, s1, 16, y16=b["d1b"])
        c("head", b["d1b"], 16, None, 0, s1, 1, y32=b["out"], residual=b["res"], relu=False)
        return b["out"]

    def loss_and_grad(self, target_norm):
        """MSE against target_norm (D, H, W f32); writes the output gradient; returns the
        device loss tensor (accumulated until zero_grad)."""
        b = self._grad_buf(tuple(target_norm.shape))
        check(lib().iane_gb_cnn_mse(_p(b["out"]), _p(target_norm), target_norm.numel(), _p(b["g_out"]), _p(b["loss"]),
                                    self._stream()))
        return b["loss"]

    def backward(self, shape):
        """Accumulate parameter gradients for the last forward (its output gradient set by
        loss_and_grad)."""
        b = self._grad_buf(tuple(shape))
        s1 = tuple(shape)
        s2 = tuple(v // 2 for v in shape)
        s3 = tuple(v // 4 for v in shape)
        f = self._flips()
        c = self._conv
        st = self._stream()
        vol1 = s1[0] * s1[1] * s1[2]
        vol2 = s2[0] * s2[1] * s2[2]
        # head (16 -> 1, no activation)
        self._wgrad(b, b["d1b"], 16, None, 0, s1, b["g_out"], 1, "head")
        c(b["g_out"], 1, None, 0, s1, f["head"], None, 16, y16=b["g16a"], relu=False, mask=b["d1b"])
        # d1b, d1a
        self._wgrad(b, b["d1a"], 16, None, 0, s1, b["g16a"], 16, "d1b")
        c(b["g16a"], 16, None, 0, s1, f["d1b"], None, 16, y16=b["g16b"], relu=False, mask=b["d1a"])
        self._wgrad(b, b["u1"], 32, b["e1b"], 16, s1, b["g16b"], 16, "d1a")
        c(b["g16b"], 16, None, 0, s1, f["d1a"], None, 48, y16=b["g_cat1"], relu=False)
        g_cat1 = b["g_cat1"].view(-1)
        # up1 -> d2b
        check(lib().iane_gb_cnn_up2_grad(_p(b["g_cat1"]), 32, *s2, _p(b["g32a"]), _p(b["d2b"]), st))
        self._wgrad(b, b["d2a"], 32, None, 0, s2, b["g32a"], 32, "d2b")
        c(b["g32a"], 32, None, 0, s2, f["d2b"], None, 32, y16=b["g32b"], relu=False, mask=b["d2a"])
        self._wgrad(b, b["u2"], 64, b["e2b"], 32, s2, b["g32b"], 32, "d2a")
        fd2a = f["d2a"]
        g_cat2 = b["g_cat2"].view(-1)
        c(b["g32b"], 32, None, 0, s2, fd2a[: 64 * 32 * 27], None, 64, y16=g_cat2[: 64 * vol2], relu=False)
        c(b["g32b"], 32, None, 0, s2, fd2a[64 * 32 * 27:], None, 32, y16=g_cat2[64 * vol2:], relu=False)
        # up2 -> e3c, e3b, e3a
        check(lib().iane_gb_cnn_up2_grad(_p(g_cat2[: 64 * vol2]), 64, *s3, _p(b["g64a"]), _p(b["e3c"]), st))
        self._wgrad(b, b["e3b"], 64, None, 0, s3, b["g64a"], 64, "e3c")
        c(b["g64a"], 64, None, 0, s3, f["e3c"], None, 64, y16=b["g64b"], relu=False, mask=b["e3b"])
        self._wgrad(b, b["e3a"], 64, None, 0, s3, b["g64b"], 64, "e3b")
        c(b["g64b"], 64, None, 0, s3, f["e3b"], None, 64, y16=b["g64a"], relu=False, mask=b["e3a"])
        self._wgrad(b, b["p2"], 32, None, 0, s3, b["g64a"], 64, "e3a")
        c(b["g64a"], 64, None, 0, s3, f["e3a"], None, 32, y16=b["g_p2"], relu=False)
        # pool2 -> e2b (adds the skip gradient already in g_cat2[64:96], ReLU mask)
        g_e2b = g_cat2[64 * vol2:]
        check(lib().iane_gb_cnn_pool2_grad(_p(b["g_p2"]), 32, *s2, _p(g_e2b), _p(b["e2b"]), 1, st))
        self._wgrad(b, b["e2a"], 32, None, 0, s2, g_e2b, 32, "e2b")
        c(g_e2b, 32, None, 0, s2, f["e2b"], None, 32, y16=b["g32a"], relu=False, mask=b["e2a"])
        self._wgrad(b, b["p1"], 16, None, 0, s2, b["g32a"], 32, "e2a")
        c(b["g32a"], 32, None, 0, s2, f["e2a"], None, 16, y16=b["g_p1"], relu=False)
        # pool1 -> e1b (skip gradient in g_cat1[32:48])
        g_e1b = g_cat1[32 * vol1:]
        check(lib().iane_gb_cnn_pool2_grad(_p(b["g_p1"]), 16, *s1, _p(g_e1b), _p(b["e1b"]), 1, st))
        self._wgrad(b, b["e1a"], 16, None, 0, s1, g_e1b, 16, "e1b")
        c(g_e1b, 16, None, 0, s1, f["e1b"], None, 16, y16=b["g16a"], relu=False, mask=b["e1a"])
        self._wgrad(b, b["x16"], 2, None, 0, s1, b["g16a"], 16, "e1a")

    def zero_grad(self):
        self.grad.zero_()
        for b in self._buffers.values():
            b["loss"].zero_()

    def step(self, lr: float = 1e-3, grad_scale: float = 1.0):
        self.steps += 1
        check(lib().iane_gb_cnn_adam(_p(self.master), _p(self.p16), _p(self.grad), _p(self.m), _p(self.v), self.size,
                                     ctypes.c_float(lr), ctypes.c_float(0.9), ctypes.c_float(0.999),
                                     ctypes.c_float(1e-8), self.steps, ctypes.c_float(grad_scale), self._stream()))
        self._flipped = None
        self._packed = None

    # -- warm start ---------------------------------------------------------------------------
    def warm_start(self, observed, sigma: float, epsilon: float = 1e-6):
        """RL start for `observed` (f32 CUDA tensor, extents multiples of 4): mean * max(net, 1e-3),
        the network run on the tensor-core kernels."""
        mean = observed.double().mean().float().clamp_min(epsilon)
        out = self.forward(observed / mean, sigma, tensor_cores=True)[0]
        return (out.clamp_min(1e-3) * mean).contiguous()

    # -- weights file: magic, version, count, then little-endian f32 master parameters ---------
    def save(self, path):
        data = self.master.cpu().numpy().astype("<f4").tobytes()
        Path(path).write_bytes(MAGIC + struct.pack("<II", 1, self.size) + data)

    def load(self, path):
        raw = Path(path).read_bytes()
        if raw[:8] != MAGIC:
            raise ValueError("not a warm-start weights file")
        version, n = struct.unpack("<II", raw[8:16])
        if version != 1 or n != self.size:
            raise ValueError("weights file does not match this network")
        host = np.frombuffer(raw[16:16 + 4 * n], dtype="<f4").astype(np.float32)
        self.master.copy_(self.torch.from_numpy(host.copy()).to(self.device))
        self.p16.copy_(self.master.to(self.torch.bfloat16))
        self._flipped = None
        self._packed = None


# ---------------------------------------------------------------------------------------------
# training data


def phantom(rng, shape, count, radius=(2.0, 20.0), intensity=(50.0, 1000.0), background=10.0, device="cuda"):
    """Ellipsoid phantom on the device: `count` axis-aligned ellipsoids with radii and
    intensities uniform in the given ranges on a constant background (the generator of the
    256x256x64 deconvolution benchmark, at any shape). shape = (D, H, W)."""
    import torch

    dev = torch.device(device)
    z, y, x = torch.meshgrid(*[torch.arange(n, dtype=torch.float32, device=dev) for n in shape], indexing="ij")
    vol = torch.full(shape, background, dtype=torch.float32, device=dev)
    for _ in range(count):
        c = [rng.uniform(0, n) for n in shape]
        r = [rng.uniform(*radius) for _ in shape]
        value = float(rng.uniform(*intensity))
        inside = ((z - c[0]) / r[0]) ** 2 + ((y - c[1]) / r[1]) ** 2 + ((x - c[2]) / r[2]) ** 2 <= 1.0
        vol += value * inside
    return vol


def psf_extent(sigma: float) -> int:
    return 2 * int(np.ceil(2.5 * sigma)) + 1


def observe(truth, sigma, peak, seed, device="cuda"):
    """Blur `truth` with the normalised isotropic Gaussian PSF of width `sigma` (zero border),
    scale the blurred image to maximum `peak` and draw Poisson counts. Returns (observed,
    psf, scale) with observed ~ Poisson(scale * (truth * psf))."""
    import torch

    from . import synth

    k = psf_extent(sigma)
    psf = torch.from_numpy(synth.gaussian_psf((k, k, k), (sigma, sigma, sigma))).to(truth.device)
    blurred = torch.empty_like(truth)
    convolve(truth, psf, blurred, "zero")
    scale = peak / float(blurred.max())
    blurred *= scale
    gen = torch.Generator(device=truth.device)
    gen.manual_seed(int(seed))
    return torch.poisson(blurred, generator=gen), psf, scale


def make_pair(rng, size=64, iterations=200, device="cuda", ellipsoids=16, sigma_range=(1.0, 3.0),
              peak_range=(100.0, 2000.0)):
    """One training pair (observed, sigma, target, psf): an ellipsoid phantom of size^3 voxels,
    an isotropic Gaussian PSF with sigma uniform in `sigma_range`, Poisson counts with peak
    uniform in `peak_range`, and the `iterations`-iteration FP32 Richardson-Lucy result from
    the flat start mean(observed)."""
    import torch

    truth = phantom(rng, (size, size, size), ellipsoids, device=device)
    sigma = float(rng.uniform(*sigma_range))
    observed, psf, _ = observe(truth, sigma, float(rng.uniform(*peak_range)), rng.integers(0, 2 ** 31), device)
    rl = RichardsonLucy(psf, observed.shape)
    target = torch.empty_like(observed)
    rl.run(observed, target, iterations, 1e-6, init=rl.INIT_MEAN)
    rl.close()
    return observed, sigma, target, psf


def train(net: WarmStartNet, pairs, epochs=4, lr=2e-3, log=None, seed=0):
    """Adam on the MSE between the net output and target / mean(observed), one volume per
    step, pairs shuffled every epoch, learning rate halved twice over the run."""
    rng = np.random.default_rng(seed)
    losses = []
    steps = epochs * len(pairs)
    step = 0
    for epoch in range(epochs):
        running = 0.0
        for i in rng.permutation(len(pairs)):
            observed, sigma, target, _ = pairs[i]
            mean = observed.double().mean().float().clamp_min(1e-6)
            net.zero_grad()
            net.forward(observed / mean, sigma)
            loss = net.loss_and_grad((target / mean).contiguous())
            net.backward(tuple(observed.shape))
            net.step(lr=lr * 0.25 ** (step / max(1, steps)))
            step += 1
            if step % 256 == 0 or step == steps:
                running = float(loss.item())
                losses.append(running)
                if log:
                    log(f"epoch {epoch} step {step} loss {running:.4e}")
    return losses


# ---------------------------------------------------------------------------------------------
# evaluation: plain FP32 RL from the flat start against the learned start + BF16 RL


def _rel_l2(a, b) -> float:
    return float((a.double() - b.double()).norm() / b.double().norm())


def poisson_deviance(observed, estimate, psf, epsilon: float = 1e-6) -> float:
    """2 * sum(o log(o / p) - (o - p)) with p = max(estimate (*) psf, eps) (zero border), the
    negative Poisson log-likelihood up to a constant: the objective every RL iteration lowers."""
    import torch

    pred = torch.empty_like(estimate)
    convolve(estimate, psf, pred, "zero")
    p = pred.double().clamp_min(epsilon)
    o = observed.double()
    term = torch.where(o > 0, o * torch.log(o / p), torch.zeros_like(p)) - (o - p)
    return float(2.0 * term.sum())


def data_residual(observed, estimate, psf) -> float:
    """||estimate (*) psf - observed|| / ||observed|| (zero border)."""
    pred = estimate.new_empty(estimate.shape)
    convolve(estimate, psf, pred, "zero")
    return float((pred.double() - observed.double()).norm() / observed.double().norm())


def evaluate(net: WarmStartNet, seed=7, sigma=2.0, peak=1000.0, tolerance=1e-3, reference_iterations=200,
             max_iterations=400, repeats=3, device="cuda", log=None):
    """The 256x256x64 ellipsoid volume (200 ellipsoids, radii 2-20) blurred by the isotropic
    Gaussian PSF of width `sigma`, Poisson counts with peak `peak`. Reference: the
    `reference_iterations`-iteration FP32 RL result from the flat start. Three stopping rules:

    * "residual": iterate until the data fit is as good as the reference's -- the Poisson
      deviance of the estimate (RL's own objective) within `tolerance` (relative) of the
      reference's deviance. Plain RL from the flat start is the judge: a warm start counts
      when RL from it reaches the residual tolerance that plain RL reaches;
    * "to_reference": iterate until rel-L2(estimate, reference) <= tolerance;
    * "converged": iterate until the relative L2 change of one iteration <= tolerance.

    For each rule and arm (plain = FP32 RL from the flat start; learned = network start +
    BF16 tensor-core RL) the iteration count, the wall time (CUDA events, median of
    `repeats`) and the final errors against the reference and the truth. Returns a dict."""
    import torch

    from . import synth

    dev = torch.device(device)
    truth_np = synth.ellipsoid_phantom((256, 256, 64), 200, seed=seed)
    truth = torch.from_numpy(truth_np).to(dev)
    observed, psf, scale = observe(truth, sigma, peak, seed + 1, device)
    truth = truth * scale
    shape = tuple(observed.shape)
    rl32 = RichardsonLucy(psf, shape)
    rl16 = RichardsonLucy(psf, shape, precision="bf16")
    s32 = torch.empty(rl32.scratch_bytes, dtype=torch.uint8, device=dev)
    s16 = torch.empty(rl16.scratch_bytes, dtype=torch.uint8, device=dev)
    reference = torch.empty_like(observed)
    rl32.run(observed, reference, reference_iterations, 1e-6, init=rl32.INIT_MEAN, scratch=s32)

    target_dev = poisson_deviance(observed, reference, psf)

    def trajectory(rl, scratch, start):
        """errors[k] = rel-L2 vs reference after k iterations (k = 0 is the start); changes[k]
        = relative change of iteration k; excess[k] = deviance / reference deviance - 1."""
        est = torch.empty_like(observed)
        if start is None:
            est.fill_(float(observed.double().mean().clamp_min(1e-6)))
        else:
            est.copy_(start)
        errors, changes = [_rel_l2(est, reference)], [float("nan")]
        excess = [poisson_deviance(observed, est, psf) / target_dev - 1.0]
        stats = torch.zeros(2, dtype=torch.float64, device=dev)
        for k in range(max_iterations):
            init = rl.INIT_MEAN if start is None and k == 0 else rl.INIT_GIVEN
            rl.run(observed, est, 1, 1e-6, init=init, scratch=scratch, stats=stats)
            errors.append(_rel_l2(est, reference))
            changes.append(float(stats[1].item()))
            excess.append(poisson_deviance(observed, est, psf) / target_dev - 1.0)
            if errors[-1] <= tolerance and changes[-1] <= tolerance and excess[-1] <= tolerance:
                break
        return errors, changes, excess, est

    def first(values, tol):
        for k, v in enumerate(values):
            if k > 0 and v <= tol:
                return k
        return None

    def timed(fn):
        times = []
        for _ in range(repeats + 1):
            torch.cuda.synchronize()
            a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            a.record()
            fn()
            b.record()
            torch.cuda.synchronize()
            times.append(a.elapsed_time(b))
        return float(np.median(times[1:]))

    e_plain, c_plain, x_plain, _ = trajectory(rl32, s32, None)
    start = net.warm_start(observed, sigma)
    torch.cuda.synchronize()
    e_learn, c_learn, x_learn, _ = trajectory(rl16, s16, start)
    out = {"volume": [256, 256, 64], "psf": [psf_extent(sigma)] * 3, "sigma": sigma, "peak": peak,
           "tolerance": tolerance, "reference_iterations": reference_iterations,
           "reference_deviance": target_dev, "reference_data_residual": data_residual(observed, reference, psf),
           "start_error": {"flat": e_plain[0], "learned": e_learn[0]},
           "start_deviance_excess": {"flat": x_plain[0], "learned": x_learn[0]}}
    est = torch.empty_like(observed)

    def plain(n):
        return lambda: rl32.run(observed, est, n, 1e-6, init=rl32.INIT_MEAN, scratch=s32)

    def learned(n):
        def fn():
            s = net.warm_start(observed, sigma)
            if n:
                rl16.run(observed, s, n, 1e-6, init=rl16.INIT_GIVEN, scratch=s16)
        return fn

    net_ms = timed(learned(0))
    out["network_ms"] = net_ms
    for rule, p_vals, l_vals in (("residual", x_plain, x_learn), ("to_reference", e_plain, e_learn),
                                 ("converged", c_plain, c_learn)):
        n0, n1 = first(p_vals, tolerance), first(l_vals, tolerance)
        r = {"plain_iterations": n0, "learned_iterations": n1}
        if n0 is not None:
            r["plain_ms"] = timed(plain(n0))
            r["plain_error"] = e_plain[n0]
            r["plain_deviance_excess"] = x_plain[n0]
        if n1 is not None:
            r["learned_ms"] = timed(learned(n1))
            r["learned_error"] = e_learn[n1]
            r["learned_deviance_excess"] = x_learn[n1]
        else:
            vals = e_learn if rule != "residual" else x_learn
            r["learned_min"] = min(vals)
            r["learned_min_at"] = int(np.argmin(vals))
        if n0 is not None and n1 is not None:
            r["speedup"] = r["plain_ms"] / r["learned_ms"]
        out[rule] = r
    # quality against the truth at the converged stopping points
    rc = out["converged"]
    for arm, rl, scratch, n, start_fn in (("plain", rl32, s32, rc["plain_iterations"], None),
                                         ("learned", rl16, s16, rc["learned_iterations"], True)):
        if n is None:
            continue
        if start_fn is None:
            rl.run(observed, est, n, 1e-6, init=rl.INIT_MEAN, scratch=scratch)
        else:
            est.copy_(net.warm_start(observed, sigma))
            rl.run(observed, est, n, 1e-6, init=rl.INIT_GIVEN, scratch=scratch)
        rc[arm + "_truth_error"] = _rel_l2(est, truth)
    out["reference_truth_error"] = _rel_l2(reference, truth)
    rl32.close()
    rl16.close()
    if log:
        log(out)
    return out


DEFAULT_WEIGHTS = Path(__file__).resolve().parent / "weights" / "warm_start_3d.bin"


def load_default(device="cuda") -> WarmStartNet:
    """The network with the weights shipped in the package."""
    net = WarmStartNet(device)
    net.load(DEFAULT_WEIGHTS)
    return net


def main(argv=None):
    import argparse
    import json
    import time

    import torch

    ap = argparse.ArgumentParser(description="train or evaluate the Richardson-Lucy warm-start network")
    sub = ap.add_subparsers(dest="cmd", required=True)
    t = sub.add_parser("train")
    t.add_argument("--volumes", type=int, default=4096)
    t.add_argument("--size", type=int, default=64)
    t.add_argument("--epochs", type=int, default=6)
    t.add_argument("--lr", type=float, default=2e-3)
    t.add_argument("--seed", type=int, default=0)
    t.add_argument("--out", default=str(DEFAULT_WEIGHTS))
    f = sub.add_parser("forward", help="time the tensor-core forward of the shipped network")
    f.add_argument("--shape", type=int, nargs=3, default=[64, 256, 256], metavar=("D", "H", "W"))
    f.add_argument("--reps", type=int, default=3)
    f.add_argument("--simt", action="store_true", help="use the SIMT kernels instead")
    e = sub.add_parser("eval")
    e.add_argument("--weights", default=str(DEFAULT_WEIGHTS))
    e.add_argument("--seed", type=int, default=7)
    e.add_argument("--sigma", type=float, default=2.0)
    a = ap.parse_args(argv)
    torch.cuda.set_device(0)
    if a.cmd == "train":
        rng = np.random.default_rng(a.seed)
        t0 = time.time()
        pairs = [make_pair(rng, size=a.size) for _ in range(a.volumes)]
        torch.cuda.synchronize()
        print(f"generated {len(pairs)} pairs in {time.time() - t0:.1f} s", flush=True)
        net = WarmStartNet("cuda", seed=a.seed)
        t0 = time.time()
        train(net, pairs, epochs=a.epochs, lr=a.lr, log=lambda m: print(m, flush=True), seed=a.seed)
        torch.cuda.synchronize()
        print(f"trained in {time.time() - t0:.1f} s", flush=True)
        Path(a.out).parent.mkdir(parents=True, exist_ok=True)
        net.save(a.out)
    elif a.cmd == "forward":
        net = load_default("cuda")
        gen = torch.Generator(device="cuda")
        gen.manual_seed(0)
        vol = torch.rand(tuple(a.shape), generator=gen, device="cuda") * 2.0
        net.forward(vol, 2.0, tensor_cores=not a.simt)  # first call packs the weights
        torch.cuda.synchronize()
        start, stop = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        start.record()
        for _ in range(a.reps):
            net.forward(vol, 2.0, tensor_cores=not a.simt)
        stop.record()
        torch.cuda.synchronize()
        print(json.dumps({"shape": a.shape, "tensor_cores": not a.simt, "ms": start.elapsed_time(stop) / a.reps}))
    else:
        net = WarmStartNet("cuda")
        net.load(a.weights)
        print(json.dumps(evaluate(net, seed=a.seed, sigma=a.sigma)), flush=True)


if __name__ == "__main__":
    main()
