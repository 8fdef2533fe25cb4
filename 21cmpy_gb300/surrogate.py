"""Learned surrogate of the excursion-set map (density, zeta, R_mfp, T_vir, z) -> x_HI.

No counterpart in the reference.  An 8-layer 3D convolutional network (3^3 kernels, circular
padding, 32 hidden channels, ReLU, sigmoid output) whose forward and backward passes run on the
project's BF16 tensor-core kernels (``sg_conv3d_fwd`` / ``sg_conv3d_wgrad``, FP32 accumulation).
Training pairs come from the plain engine; the plain engine also measures the surrogate's error
and is its fallback (:class:`SurrogateSweep`).

Channels-last BF16 activations [n][n][n][C].  Input features (16 channels, 5 + len(smoothing)
used): normalised density delta / (4 D(z)), zeta / 80, R_mfp / 50, log10(T_vir) - 4, (z - 6) / 4,
then the density smoothed with the real-space top hat of the excursion set (the engine's own
transforms and window) at radii of 4, 8, 16 and 32 cells, scaled like channel 0.  Eight layers of
3^3 kernels see +-8 cells; the excursion set's largest radius reaches 32 cells at 128^3 / 200 Mpc,
and the smoothed channels hand the network that large-scale information directly.
"""
from __future__ import annotations

import ctypes as C
import math
from dataclasses import dataclass

import numpy as np
import torch

from . import _lib, cosmology, schedule

LAYERS = [(16, 32)] + [(32, 32)] * 6 + [(32, 16)]      # (cin, cout); last: channel 0 is x_HI
SMOOTH_CELLS = (4.0, 8.0, 16.0, 32.0)                 # radii (cells) of the smoothed input channels
PARAM_RANGES = {"zeta": (10.0, 80.0), "R_max": (5.0, 50.0), "log10_tvir": (4.0, 5.3), "z": (6.0, 10.0)}


def _p(t):
    return C.c_void_p(t.data_ptr()) if t is not None else C.c_void_p()


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


class SurrogateNet:
    """Weights (FP32 masters) and the BF16 tensor-core forward / backward passes."""

    def __init__(self, device=None, seed: int = 0, smoothing=SMOOTH_CELLS):
        self.lib = _lib.load()
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.smoothing = tuple(float(r) for r in smoothing)
        if len(self.smoothing) > 11:
            raise ValueError("at most 11 smoothed input channels")
        self.n_in = 5 + len(self.smoothing)
        g = torch.Generator(device="cpu").manual_seed(seed)
        self.w, self.b = [], []
        for li, (cin, cout) in enumerate(LAYERS):
            used_in = self.n_in if li == 0 else cin
            std = math.sqrt(2.0 / (27 * used_in))
            w = torch.randn((27, cout, cin), generator=g) * std
            if li == 0:
                w[:, :, self.n_in:] = 0.0
            if li == len(LAYERS) - 1:
                w[:, 1:, :] = 0.0
                w *= 0.5
            self.w.append(w.to(self.device).requires_grad_(False))
            self.b.append(torch.zeros(cout, device=self.device))
        self._ws = None
        self._wb, self._wb_key = None, None

    def parameters(self):
        return self.w + self.b

    def check(self):
        """Synchronises; raises if a tcgen05 convolution gave up a bounded wait since the last check."""
        _lib.check("sg_check", self.lib.sg_check(), self.lib)

    def load_state(self, state):
        if tuple(state.get("smoothing", ())) != self.smoothing:
            raise ValueError(f"weights were trained with smoothing {state.get('smoothing', ())}, "
                             f"this network uses {self.smoothing}")
        for i, (w, b) in enumerate(zip(state["w"], state["b"])):
            self.w[i].copy_(w)
            self.b[i].copy_(b)

    def state(self):
        return {"w": [w.detach().cpu() for w in self.w], "b": [b.detach().cpu() for b in self.b],
                "smoothing": self.smoothing}

    def features(self, delta: torch.Tensor, z: float, zeta: float, R_max: float, t_vir: float,
                 cosmo=cosmology.BASELINE_COSMO) -> torch.Tensor:
        """This network's input for a density box (with its smoothed channels)."""
        return features(delta, z, zeta, R_max, t_vir, cosmo, smoothing=self.smoothing)

    # ------------------------------------------------------------------ kernels
    def _conv(self, n, cin, cout, mode, x, w, bias, out, mask=None):
        rc = self.lib.sg_conv3d_fwd(n, cin, cout, mode, _p(x), _p(w), _p(bias), _p(out), _p(mask), _stream())
        _lib.check("sg_conv3d_fwd", rc, self.lib)

    def _wgrad(self, n, cin, cout, x, dz, dw, db):
        need = int(self.lib.sg_conv3d_wgrad_workspace(n, cin, cout))
        if self._ws is None or self._ws.numel() * 4 < need:
            self._ws = torch.empty(need // 4 + 1, dtype=torch.float32, device=self.device)
        rc = self.lib.sg_conv3d_wgrad(n, cin, cout, _p(x), _p(dz), _p(dw), _p(db), _p(self._ws), need, _stream())
        _lib.check("sg_conv3d_wgrad", rc, self.lib)

    def bf16_weights(self):
        """BF16 copies of the FP32 master weights, converted again only after a weight changed (in
        place, as the optimiser and load_state change them: tracked by the tensors' versions)."""
        key = tuple((w.data_ptr(), w._version) for w in self.w)
        if self._wb_key != key:
            self._wb = [w.to(torch.bfloat16).contiguous() for w in self.w]
            self._wb_key = key
        return self._wb

    def forward(self, feats: torch.Tensor, keep: bool = False):
        """feats: bf16 [n, n, n, 16].  Returns (x_HI float [n, n, n], activations if keep)."""
        n = feats.shape[0]
        acts = [feats]
        x = feats
        wb = self.bf16_weights()
        for li, (cin, cout) in enumerate(LAYERS[:-1]):
            y = torch.empty((n, n, n, cout), dtype=torch.bfloat16, device=self.device)
            self._conv(n, cin, cout, 0, x, wb[li], self.b[li], y)
            acts.append(y)
            x = y
        out = torch.empty((n, n, n), dtype=torch.float32, device=self.device)
        cin, cout = LAYERS[-1]
        self._conv(n, cin, cout, 1, x, wb[-1], self.b[-1], out)
        return out, (acts if keep else None)

    def backward(self, acts, pred: torch.Tensor, target: torch.Tensor):
        """Gradients of the summed binary cross-entropy; returns (dW list, db list)."""
        n = pred.shape[0]
        L = len(LAYERS)
        dz = torch.zeros((n, n, n, LAYERS[-1][1]), dtype=torch.bfloat16, device=self.device)
        dz[..., 0] = (pred - target).to(torch.bfloat16)          # d(BCE)/d(logit), summed loss
        dws, dbs = [None] * L, [None] * L
        for li in range(L - 1, -1, -1):
            cin, cout = LAYERS[li]
            dw = torch.empty((27, cout, cin), dtype=torch.float32, device=self.device)
            db = torch.empty(cout, dtype=torch.float32, device=self.device)
            self._wgrad(n, cin, cout, acts[li], dz, dw, db)
            dws[li], dbs[li] = dw, db
            if li > 0:
                wflip = self.w[li].flip(0).transpose(1, 2).contiguous().to(torch.bfloat16)   # [27][cin][cout]
                dprev = torch.empty((n, n, n, cin), dtype=torch.bfloat16, device=self.device)
                self._conv(n, cout, cin, 2, dz, wflip, None, dprev, mask=acts[li])
                dz = dprev
        # frozen entries: unused input channels of layer 0, unused outputs of the last layer
        dws[0][:, :, self.n_in:] = 0.0
        dws[-1][:, 1:, :] = 0.0
        dbs[-1][1:] = 0.0
        return dws, dbs


_smooth_plans = {}


def smoothed_fields(delta: torch.Tensor, radii_cells) -> torch.Tensor:
    """The density smoothed with the real-space top hat W(kR) at each radius (in cells): one forward
    transform, then per radius the window (``ic_shape``, the excursion set's filter) and an inverse
    transform, all on the engine's kernels.  Returns float32 [len(radii), n, n, n]."""
    from .engine import ExcursionSetPlan
    n = delta.shape[0]
    key = (n, str(delta.device))
    if key not in _smooth_plans:
        _smooth_plans[key] = ExcursionSetPlan(n, float(n), max_radii=1, device=delta.device)   # lengths in cells
    plan = _smooth_plans[key]
    lib = _lib.load()
    out = torch.empty((len(radii_cells), n, n, n), dtype=torch.float32, device=delta.device)
    with torch.cuda.device(delta.device):
        X = plan.fft_r2c(delta)
        Y = torch.empty_like(X)
        for j, R in enumerate(radii_cells):
            rc = lib.ic_shape(n, C.c_float(float(n)), _p(X), -1, 0, C.c_float(float(R)), 0, _p(Y), _stream())
            _lib.check("ic_shape", rc, lib)
            out[j] = plan.fft_c2r(Y)
        out *= 1.0 / float(n) ** 3
    return out


def features(delta: torch.Tensor, z: float, zeta: float, R_max: float, t_vir: float,
             cosmo=cosmology.BASELINE_COSMO, smoothing=SMOOTH_CELLS) -> torch.Tensor:
    """bf16 [n, n, n, 16] network input for a density box at redshift z and a parameter point:
    density, the four parameters, and the density smoothed at the radii `smoothing` (cells)."""
    n = delta.shape[0]
    if not (isinstance(delta, torch.Tensor) and delta.is_cuda and delta.dtype == torch.float32
            and delta.is_contiguous() and tuple(delta.shape) == (n, n, n)):
        raise ValueError("delta must be a contiguous float32 (n, n, n) CUDA tensor")
    const = torch.zeros(16, dtype=torch.float32)
    const[1:5] = torch.tensor([zeta / 80.0, R_max / 50.0, math.log10(t_vir) - 4.0, (z - 6.0) / 4.0])
    bits = (C.c_uint16 * 16)(*[int(v) & 0xFFFF for v in const.to(torch.bfloat16).view(torch.int16).tolist()])
    scale = float(np.float32(1.0 / (4.0 * cosmology.growth_factor(z, cosmo))))
    f = torch.empty((n, n, n, 16), dtype=torch.bfloat16, device=delta.device)
    lib = _lib.load()
    smoothing = tuple(smoothing)
    with torch.cuda.device(delta.device):
        if smoothing:
            sm = smoothed_fields(delta, smoothing)
            rc = lib.sg_features_ms(n, _p(delta), _p(sm), len(smoothing), C.c_float(scale), bits, _p(f), _stream())
            _lib.check("sg_features_ms", rc, lib)
        else:
            rc = lib.sg_features(n, _p(delta), C.c_float(scale), bits, _p(f), _stream())
            _lib.check("sg_features", rc, lib)
    return f


class Adam:
    """Adam on the FP32 master weights (elementwise updates)."""

    def __init__(self, params, lr=1e-3, betas=(0.9, 0.999), eps=1e-8):
        self.params = params
        self.lr, self.b1, self.b2, self.eps = lr, betas[0], betas[1], eps
        self.m = [torch.zeros_like(p) for p in params]
        self.v = [torch.zeros_like(p) for p in params]
        self.t = 0

    def step(self, grads, scale: float = 1.0):
        self.t += 1
        c1 = 1 - self.b1 ** self.t
        c2 = 1 - self.b2 ** self.t
        for p, g, m, v in zip(self.params, grads, self.m, self.v):
            g = g * scale
            m.mul_(self.b1).add_(g, alpha=1 - self.b1)
            v.mul_(self.b2).addcmul_(g, g, value=1 - self.b2)
            p.sub_(self.lr * (m / c1) / ((v / c2).sqrt() + self.eps))


@dataclass
class Sample:
    delta: torch.Tensor          # float32 [n, n, n] on the device
    xH: torch.Tensor             # float32 [n, n, n] plain-engine target
    z: float
    zeta: float
    R_max: float
    t_vir: float


def draw_params(rng: np.random.Generator):
    return dict(zeta=float(rng.uniform(*PARAM_RANGES["zeta"])), R_max=float(rng.uniform(*PARAM_RANGES["R_max"])),
                t_vir=float(10 ** rng.uniform(*PARAM_RANGES["log10_tvir"])), z=float(rng.uniform(*PARAM_RANGES["z"])))


class DataGenerator:
    """Training / evaluation pairs at n^3: GPU Gaussian random fields through the engine's FFT and
    x_HI labels from the plain engine."""

    def __init__(self, n: int = 128, box_len: float = 200.0, cosmo=cosmology.BASELINE_COSMO, device=None):
        from .engine import ExcursionSetPlan
        from .autotune import ensure_tuned
        self.n, self.box_len, self.cosmo = n, box_len, cosmo
        self.device = torch.device(device) if device is not None else torch.device("cuda", torch.cuda.current_device())
        self.plan = ExcursionSetPlan(n, box_len, max_radii=96, device=self.device)
        ensure_tuned(self.plan)
        self.amp = self._amplitude()
        self.table = cosmology.sigma_table(cosmo)

    def _amplitude(self):
        n, L = self.n, self.box_len
        dk = 2 * math.pi / L
        kz = np.fft.fftfreq(n, d=1.0 / n) * dk
        kx = np.fft.rfftfreq(n, d=1.0 / n) * dk
        k = np.sqrt(kz[:, None, None] ** 2 + kz[None, :, None] ** 2 + kx[None, None, :] ** 2)
        a = np.zeros_like(k)
        nz = k > 0
        a[nz] = np.sqrt(cosmology.power_spectrum_z0(k[nz], self.cosmo) * n ** 3 / L ** 3)
        return torch.from_numpy(a.astype(np.float32)).to(self.device)

    def density(self, seed: int, z: float) -> torch.Tensor:
        """Linear density at z of GRF realisation `seed` (white noise from a seeded torch generator)."""
        n = self.n
        g = torch.Generator(device=self.device).manual_seed(int(seed))
        white = torch.randn((n, n, n), generator=g, device=self.device, dtype=torch.float32)
        W = self.plan.fft_r2c(white)
        W *= self.amp
        d = self.plan.fft_c2r(W) / float(n) ** 3
        return (d * cosmology.growth_factor(z, self.cosmo)).contiguous()

    def sample(self, seed: int, params: dict) -> Sample:
        d = self.density(seed, params["z"])
        st = schedule.ionize_setup(self.n, self.box_len, params["z"], zeta=params["zeta"],
                                   t_vir_min=params["t_vir"], R_max=params["R_max"], cosmo=self.cosmo,
                                   table=self.table)
        xh, _ = self.plan.run(d, st)
        return Sample(d, xh.clone(), params["z"], params["zeta"], params["R_max"], params["t_vir"])


def train(net: SurrogateNet, samples, epochs: int = 1, lr: float = 3e-4, log=None):
    """Adam over the pairs, one box per step; returns the per-step mean BCE.

    Step sizes of 2e-3 and above saturate the sigmoid within the first epoch (every output pinned at
    0 or 1, BCE ~ 9.6); 3e-4 converges on 32^3 and 128^3 pairs."""
    opt = Adam(net.parameters(), lr=lr)
    losses = []
    for ep in range(epochs):
        for s in samples:
            f = net.features(s.delta, s.z, s.zeta, s.R_max, s.t_vir)
            pred, acts = net.forward(f, keep=True)
            dws, dbs = net.backward(acts, pred, s.xH)
            nvox = float(s.delta.numel())
            opt.step(dws + dbs, scale=1.0 / nvox)
            p = pred.clamp(1e-6, 1 - 1e-6)
            loss = -(s.xH * torch.log(p) + (1 - s.xH) * torch.log(1 - p)).mean()
            losses.append(loss)
        net.check()
        if log:
            log(f"epoch {ep}: mean BCE {torch.stack(losses[-len(samples):]).mean().item():.4f}")
    return torch.stack(losses).cpu().numpy() if losses else np.zeros(0)


def evaluate(net: SurrogateNet, samples, plan=None, k_range=(0.1, 1.0), num_bins: int = 20):
    """Surrogate vs plain engine: mean |dx_HI|, flag agreement at 0.5, P21(k) ratio on k_range."""
    errs, agree, ratios = [], [], []
    for s in samples:
        f = net.features(s.delta, s.z, s.zeta, s.R_max, s.t_vir)
        pred, _ = net.forward(f)
        errs.append((pred - s.xH).abs().mean().item())
        agree.append(((pred >= 0.5) == (s.xH >= 0.5)).float().mean().item())
        if plan is not None:
            c = cosmology.brightness_temperature_factor(s.z, cosmology.BASELINE_COSMO)
            edges = schedule.pk_edges(plan.n, plan.box_len, num_bins)
            pk = []
            for xh in (pred, s.xH):
                dT, ave = plan.delta_T(xh.contiguous(), s.delta, c)
                pk.append(plan.power_spectrum(dT, ave, edges).cpu().numpy())
            kav = pk[1][1]
            sel = (kav >= k_range[0]) & (kav <= k_range[1]) & (pk[1][0] > 0)
            ratios.append(pk[0][0][sel] / pk[1][0][sel])
    r = np.concatenate(ratios) if ratios else np.zeros(0)
    return {"mean_abs_dxHI": float(np.mean(errs)), "flag_agreement": float(np.mean(agree)),
            "p21_ratio_median": float(np.median(r)) if r.size else None,
            "p21_ratio_max_dev": float(np.max(np.abs(r - 1))) if r.size else None,
            "p21_within_10pct": float(np.mean(np.abs(r - 1) <= 0.1)) if r.size else None}


class SurrogateSweep:
    """Parameter sweeps with the surrogate and the plain engine as fallback and judge.

    Every `check_every`-th point runs both the surrogate and the plain engine and records the
    surrogate's mean |dx_HI| there; a checked point over `max_abs_err` returns the engine's box.
    Between checks the surrogate serves the points while the mean error over all checked points is
    within `max_abs_err`, and the plain engine serves them otherwise; checks go on in both states,
    so trust lost to an unlucky check comes back.  Points outside the training ranges always run the
    engine.
    """

    def __init__(self, net: SurrogateNet, gen: DataGenerator, max_abs_err: float = 0.05, check_every: int = 16):
        self.net, self.gen = net, gen
        self.max_abs_err, self.check_every = max_abs_err, check_every
        self.calls = 0
        self.fallbacks = 0
        self.checked = []

    @property
    def trusted(self) -> bool:
        return not self.checked or float(np.mean(self.checked)) <= self.max_abs_err

    def in_range(self, params):
        lo, hi = PARAM_RANGES["log10_tvir"]
        return (PARAM_RANGES["zeta"][0] <= params["zeta"] <= PARAM_RANGES["zeta"][1]
                and PARAM_RANGES["R_max"][0] <= params["R_max"] <= PARAM_RANGES["R_max"][1]
                and lo <= math.log10(params["t_vir"]) <= hi
                and PARAM_RANGES["z"][0] <= params["z"] <= PARAM_RANGES["z"][1])

    def __call__(self, delta: torch.Tensor, params: dict):
        self.calls += 1
        if not self.in_range(params):
            return self._engine(delta, params), "engine"
        check = bool(self.check_every) and self.calls % self.check_every == 0
        if not check and not self.trusted:
            return self._engine(delta, params), "engine"
        pred, _ = self.net.forward(self.net.features(delta, params["z"], params["zeta"], params["R_max"], params["t_vir"]))
        if check:
            ref = self._engine(delta, params)
            err = (pred - ref).abs().mean().item()
            self.checked.append(err)
            if err > self.max_abs_err:
                return ref, "engine"
        return pred, "surrogate"

    def _engine(self, delta, params):
        self.fallbacks += 1
        st = schedule.ionize_setup(self.gen.n, self.gen.box_len, params["z"], zeta=params["zeta"],
                                   t_vir_min=params["t_vir"], R_max=params["R_max"], cosmo=self.gen.cosmo,
                                   table=self.gen.table)
        xh, _ = self.gen.plan.run(delta, st)
        return xh
