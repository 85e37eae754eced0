"""Learned initial guess for Sersic fits of 64 x 64 stamps.

No counterpart in the reference: AstroPhot starts its LM from the heuristics of
``Galaxy_Model.initialize`` / ``parametric_initialize`` (models/galaxy_model_object.py:60-113,
models/_shared_methods.py:116-166).  Here a 6-layer CNN (``ap_cnn_*`` in the C ABI, bf16
tensor-core GEMMs with fp32 accumulation) proposes the 7 Sersic parameters; the LM starts from
the proposal unless its chi^2 is worse than that of the moments initialiser
(``ap_moments_init``), which is then used instead.  LM's final chi^2 judges the outcome: a
stamp left with a poor fit is fitted again by the plain method, LM from the reference's own
heuristic initial values (``ap_reference_init``), and keeps the better of the two.

Training data come only from the library's own renderer: Sersic stamps drawn from the C0
parameter distributions (centre 32 + U(-1, 1), n ~ U(0.5, 4), Re ~ U(5, 20), q ~ U(0.3, 1),
PA ~ U(0, pi), log10 Ie ~ U(0, 2)), a flat sky of 1.0, a Moffat PSF (beta 3.5) with
FWHM ~ U(2, 5) px (64 levels, side 4 FWHM rounded to odd: 9 to 21 px) and Gaussian noise of
constant sigma set by a signal-to-noise ratio ~ U(10, 200), SNR = sqrt(sum(galaxy^2)) / sigma.
"""

from __future__ import annotations

import ctypes
import math
import os
from dataclasses import dataclass
from typing import Optional

import numpy as np
import torch

from . import _native as N
from .synthetic import moffat_rd, moffat_stamp

__all__ = ("InitNet", "StampSet", "draw_stamp_params", "psf_bank", "make_stamps", "learned_fit", "learned_fit_host",
           "plain_fit",
           "heuristic_init", "subset", "set_tensor_path", "get_tensor_path", "tc_status",
           "WEIGHTS_PATH")

# tensor-core path of the CNN GEMMs (ap_cnn_set_path)
TENSOR_PATHS = {"mma_sync": 0, "tcgen05": 1}


def set_tensor_path(name: str) -> None:
    """``"tcgen05"`` (default: TMEM accumulators, TMA-staged operands, implicit im2col at
    inference) or ``"mma_sync"`` (ldmatrix + mma.sync tiles over explicit im2col matrices)."""
    if name not in TENSOR_PATHS:
        raise ValueError(f"tensor path {name!r}: one of {sorted(TENSOR_PATHS)}")
    N.check(N.lib().ap_cnn_set_path(TENSOR_PATHS[name]), "ap_cnn_set_path")


def get_tensor_path() -> str:
    v = ctypes.c_int32(-1)
    N.check(N.lib().ap_cnn_get_path(ctypes.byref(v)), "ap_cnn_get_path")
    return {i: k for k, i in TENSOR_PATHS.items()}[v.value]


def tc_status(clear: bool = False) -> int:
    """Error code recorded by a tcgen05 kernel (0: none; 1-5: an mbarrier wait ran out)."""
    v = ctypes.c_uint32(0)
    N.check(N.lib().ap_tc_status(1 if clear else 0, ctypes.byref(v)), "ap_tc_status")
    return int(v.value)

IMG = 64
N_OUT = 8
OUT_PAD = 16
WEIGHTS_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "weights", "init_cnn.npz")


# ---- synthetic stamps ----------------------------------------------------------------------
def draw_stamp_params(rng: np.random.Generator, n: int, size: int = IMG) -> np.ndarray:
    """[n, 8] value-space vectors (F = 0: sky 1.0) from the C0 distributions."""
    p = np.zeros((n, 8))
    p[:, 0] = size / 2 + rng.uniform(-1, 1, n)
    p[:, 1] = size / 2 + rng.uniform(-1, 1, n)
    q = rng.uniform(0.3, 1.0, n)
    bad = q >= 0.999
    while bad.any():
        q[bad] = rng.uniform(0.3, 1.0, int(bad.sum()))
        bad = q >= 0.999
    p[:, 2] = q
    p[:, 3] = rng.uniform(0.0, math.pi, n)
    p[:, 4] = rng.uniform(0.5, 4.0, n)
    p[:, 5] = rng.uniform(5.0, 20.0, n)
    p[:, 6] = rng.uniform(0.0, 2.0, n)
    return p


def psf_bank(levels: int = 64, beta: float = 3.5) -> list:
    """[levels] Moffat stamps, FWHM evenly spaced on [2, 5] px, each of side odd(4 FWHM)."""
    out = []
    for fwhm in np.linspace(2.0, 5.0, levels):
        w = int(round(4 * fwhm))
        w += 1 - (w % 2)
        out.append(moffat_stamp(beta, moffat_rd(fwhm, beta), w))
    return out


@dataclass
class StampSet:
    """A batch of 64 x 64 stamps on the device (packed [n * 4096] float32)."""

    truth: np.ndarray       # [n, 8]
    data: torch.Tensor      # [n * 4096]
    weight: torch.Tensor    # [n * 4096]
    psf: torch.Tensor       # packed PSFs (batch.pack_psf layout)
    sigma: torch.Tensor     # [n]
    batch: "N.StampBatch"


def _stamp_batch(kshapes, device) -> "N.StampBatch":
    """A plan for len(kshapes) 64 x 64 stamps with these PSF shapes."""
    opts = N.make_options(profile="sersic", psf_mode="full", free_mask=0x7F, has_sky=True)
    n = len(kshapes)
    return N.StampBatch([(IMG, IMG)] * n, list(kshapes), N.scale_geometry(n), opts, device)


def make_stamps(n: int, seed: int, bank: Optional[list] = None, device="cuda", snr=(10.0, 200.0)) -> StampSet:
    """Render ``n`` stamps with the library's own kernels and add seeded Gaussian noise."""
    rng = np.random.default_rng(seed)
    truth = draw_stamp_params(rng, n)
    if bank is None:
        bank = psf_bank()
    idx = rng.integers(0, len(bank), n)
    b = _stamp_batch([bank[k].shape[::-1] for k in idx], device)
    psf = b.pack_psf([bank[k] for k in idx])
    model = b.render(torch.tensor(truth), psf)
    gal = (model - 1.0).view(n, IMG * IMG)
    s = torch.tensor(rng.uniform(snr[0], snr[1], n), dtype=torch.float32, device=device)
    sigma = torch.sqrt(torch.sum(gal.double() ** 2, dim=1)).float() / s
    gen = torch.Generator(device=device)
    gen.manual_seed(int(seed) * 7919 + 17)
    noise = torch.randn((n, IMG * IMG), generator=gen, device=device, dtype=torch.float32)
    data = (model.view(n, -1) + sigma[:, None] * noise).reshape(-1).contiguous()
    weight = (torch.ones((n, IMG * IMG), device=device) / (sigma[:, None] ** 2)).reshape(-1).contiguous()
    return StampSet(truth, data, weight, psf, sigma, b)


# ---- the network ---------------------------------------------------------------------------
def _targets(truth: torch.Tensor, lscale: torch.Tensor) -> torch.Tensor:
    """Raw regression targets [n, 8] (see ``ap_cnn_decode``)."""
    t = torch.empty((truth.shape[0], N_OUT), dtype=torch.float64, device=truth.device)
    t[:, 0] = truth[:, 0] - IMG / 2
    t[:, 1] = truth[:, 1] - IMG / 2
    t[:, 2] = truth[:, 2]
    t[:, 3] = torch.cos(2 * truth[:, 3])
    t[:, 4] = torch.sin(2 * truth[:, 3])
    t[:, 5] = torch.log(truth[:, 4])
    t[:, 6] = torch.log(truth[:, 5])
    t[:, 7] = truth[:, 6] - lscale.double()  # log10 Ie - log10 sigma
    return t


class InitNet:
    """Parameters (fp32 master + bf16 mirror), output statistics, training and inference."""

    def __init__(self, device="cuda", seed: int = 0):
        self.device = torch.device(device)
        self.lib = N.lib()
        self.count = int(self.lib.ap_cnn_param_count())
        w_off = (ctypes.c_int64 * 6)()
        b_off = (ctypes.c_int64 * 6)()
        dims = (ctypes.c_int32 * 36)()
        N.check(self.lib.ap_cnn_layer_offsets(w_off, b_off, dims), "ap_cnn_layer_offsets")
        self.w_off, self.b_off = list(w_off), list(b_off)
        self.dims = np.array(list(dims)).reshape(6, 6)
        rng = np.random.default_rng(seed)
        p = np.zeros(self.count, dtype=np.float32)
        for l in range(6):
            cin, cout, hin, hout, K, Nn = self.dims[l]
            fan_in = 9 * cin if l < 4 else K
            W = rng.normal(0.0, math.sqrt(2.0 / fan_in), size=(Nn, K)).astype(np.float32)
            if l == 0:
                W[:, 9:] = 0.0
            if l == 5:
                W *= 0.1
                W[N_OUT:] = 0.0
            p[self.w_off[l] : self.w_off[l] + Nn * K] = W.reshape(-1)
        self.params = torch.tensor(p, device=self.device)
        self.params_bf16 = torch.empty(self.count, dtype=torch.bfloat16, device=self.device)
        self._sync_bf16()
        self.mean = torch.zeros(N_OUT, dtype=torch.float32, device=self.device)
        self.std = torch.ones(N_OUT, dtype=torch.float32, device=self.device)
        self._ws = None
        self._ws_batch = 0
        self.history = []

    def _sync_bf16(self):
        N.check(self.lib.ap_cnn_to_bf16(N._ptr(self.params), N._ptr(self.params_bf16), N._stream()), "ap_cnn_to_bf16")

    def _workspace(self, batch: int):
        need = int(self.lib.ap_cnn_workspace_bytes(batch))
        if self._ws is None or self._ws.numel() < need:
            self._ws = torch.empty(need, dtype=torch.uint8, device=self.device)
        return self._ws

    # -- persistence --
    def save(self, path: str = WEIGHTS_PATH):
        os.makedirs(os.path.dirname(path), exist_ok=True)
        np.savez_compressed(path, params=self.params.cpu().numpy(), mean=self.mean.cpu().numpy(),
                            std=self.std.cpu().numpy(), history=np.array(self.history, dtype=np.float64))

    @classmethod
    def load(cls, path: str = WEIGHTS_PATH, device="cuda") -> "InitNet":
        z = np.load(path)
        net = cls(device)
        if z["params"].shape[0] != net.count:
            raise ValueError(f"{path}: {z['params'].shape[0]} parameters, the network has {net.count}")
        net.params = torch.tensor(z["params"], dtype=torch.float32, device=net.device)
        net.mean = torch.tensor(z["mean"], dtype=torch.float32, device=net.device)
        net.std = torch.tensor(z["std"], dtype=torch.float32, device=net.device)
        net.history = list(z["history"]) if "history" in z.files else []
        net._sync_bf16()
        return net

    # -- kernels --
    def prepare(self, data: torch.Tensor, sigma: torch.Tensor, n: int, sky: float = 1.0):
        x = torch.empty(n * IMG * IMG, dtype=torch.float32, device=self.device)
        lscale = torch.empty(n, dtype=torch.float32, device=self.device)
        skyv = torch.full((n,), sky, dtype=torch.float32, device=self.device)
        sg = sigma.to(self.device, torch.float32).contiguous()
        N.check(self.lib.ap_cnn_prepare(N._ptr(data), N._ptr(skyv), N._ptr(sg), n, N._ptr(x), N._ptr(lscale),
                                        N._stream()), "ap_cnn_prepare")
        return x, lscale

    def forward(self, x: torch.Tensor, n: int) -> torch.Tensor:
        if n % 16:
            raise ValueError("batches of the CNN are multiples of 16 stamps")
        ws = self._workspace(n)
        out = torch.empty((n, OUT_PAD), dtype=torch.float32, device=self.device)
        N.check(self.lib.ap_cnn_forward(N._ptr(self.params), N._ptr(self.params_bf16), N._ptr(x), n, N._ptr(out),
                                        N._ptr(ws), ws.numel(), N._stream()), "ap_cnn_forward")
        return out

    def infer(self, x: torch.Tensor, n: int) -> torch.Tensor:
        """``forward`` for inference only (no im2col matrices kept: ``backward`` may not follow)."""
        if n % 16:
            raise ValueError("batches of the CNN are multiples of 16 stamps")
        ws = self._workspace(n)
        out = torch.empty((n, OUT_PAD), dtype=torch.float32, device=self.device)
        N.check(self.lib.ap_cnn_infer(N._ptr(self.params), N._ptr(self.params_bf16), N._ptr(x), n, N._ptr(out),
                                      N._ptr(ws), ws.numel(), N._stream()), "ap_cnn_infer")
        return out

    def kept_activations(self, n: int):
        """The activations the last ``forward`` of ``n`` stamps kept in the workspace for the
        backward pass: [act of layers 1-5 as float32 [rows, N]], out [n, 16]."""
        acts = (ctypes.c_int64 * 6)()
        out_off = ctypes.c_int64()
        N.check(self.lib.ap_cnn_workspace_offsets(n, acts, ctypes.byref(out_off)), "ap_cnn_workspace_offsets")
        dims = (ctypes.c_int32 * 36)()
        wo, bo = (ctypes.c_int64 * 6)(), (ctypes.c_int64 * 6)()
        N.check(self.lib.ap_cnn_layer_offsets(wo, bo, dims), "ap_cnn_layer_offsets")
        ws = self._workspace(n)
        out = []
        for l in range(5):
            hout, nn = dims[l * 6 + 3], dims[l * 6 + 5]
            rows = n * hout * hout
            raw = ws[acts[l] : acts[l] + rows * nn * 2]
            out.append(raw.view(torch.bfloat16).float().reshape(rows, nn))
        raw = ws[out_off.value : out_off.value + n * OUT_PAD * 4]
        return out, raw.view(torch.float32).reshape(n, OUT_PAD).clone()

    def backward(self, dout: torch.Tensor, n: int) -> torch.Tensor:
        ws = self._workspace(n)
        grads = torch.empty(self.count, dtype=torch.float32, device=self.device)
        N.check(self.lib.ap_cnn_backward(N._ptr(self.params_bf16), N._ptr(dout.contiguous()), n, N._ptr(grads),
                                         N._ptr(ws), ws.numel(), N._stream()), "ap_cnn_backward")
        return grads

    def propose(self, data: torch.Tensor, sigma: torch.Tensor, n: int, sky_F: float = 0.0,
                chunk: int = 8192) -> torch.Tensor:
        """[n, 8] value-space proposals for packed 64 x 64 stamps (sky = 10^sky_F, noise sigma[n])."""
        out = torch.empty((n, 8), dtype=torch.float64, device=self.device)
        sky = 10.0**sky_F
        for s in range(0, n, chunk):
            m = min(chunk, n - s)
            mp = (m + 15) // 16 * 16
            d = data[s * IMG * IMG : (s + m) * IMG * IMG]
            sg = sigma[s : s + m]
            if mp != m:
                d = torch.cat([d, torch.full(((mp - m) * IMG * IMG,), sky, dtype=torch.float32, device=self.device)])
                sg = torch.cat([sg, torch.ones(mp - m, dtype=sg.dtype, device=sg.device)])
            x, lscale = self.prepare(d.contiguous(), sg, mp, sky)
            o = self.infer(x, mp)
            skyF = torch.full((mp,), sky_F, dtype=torch.float64, device=self.device)
            p = torch.empty((mp, 8), dtype=torch.float64, device=self.device)
            N.check(self.lib.ap_cnn_decode(N._ptr(o), N._ptr(lscale), N._ptr(self.mean), N._ptr(self.std),
                                           N._ptr(skyF), mp, N._ptr(p), N._stream()), "ap_cnn_decode")
            out[s : s + m] = p[:m]
        return out

    # -- training --
    def set_statistics(self, raw_targets: torch.Tensor):
        self.mean = raw_targets.mean(dim=0).float().contiguous()
        self.std = raw_targets.std(dim=0).clamp_min(1e-3).float().contiguous()

    def train(self, n_stamps: int = 2_000_000, batch: int = 512, chunk: int = 8192, lr: float = 1e-3,
              lr_end: float = 2e-5, warmup: int = 200, weight_decay: float = 1e-4, seed: int = 1, log_every: int = 0):
        """Adam on fresh rendered stamps (each stamp seen once)."""
        if batch % 16 or chunk % batch:
            raise ValueError("batch must be a multiple of 16 dividing chunk")
        bank = psf_bank()
        m1 = torch.zeros(self.count, dtype=torch.float32, device=self.device)
        m2 = torch.zeros_like(m1)
        grads = torch.zeros_like(m1)
        loss_d = torch.zeros(1, dtype=torch.float64, device=self.device)
        ws = self._workspace(batch)
        n_chunks = max(1, n_stamps // chunk)
        total_steps = n_chunks * (chunk // batch)
        step = 0
        losses = []
        for c in range(n_chunks):
            st = make_stamps(chunk, seed * 1_000_003 + c, bank, self.device)
            x, lscale = self.prepare(st.data, st.sigma, chunk)
            raw = _targets(torch.tensor(st.truth, device=self.device), lscale)
            if c == 0 and step == 0:
                self.set_statistics(raw)
            t = ((raw - self.mean.double()) / self.std.double()).float().contiguous()
            for b0 in range(0, chunk, batch):
                step += 1
                if step <= warmup:
                    lr_t = lr * step / warmup
                else:
                    f = (step - warmup) / max(1, total_steps - warmup)
                    lr_t = lr_end + 0.5 * (lr - lr_end) * (1 + math.cos(math.pi * min(1.0, f)))
                xb = x[b0 * IMG * IMG : (b0 + batch) * IMG * IMG]
                tb = t[b0 : b0 + batch]
                N.check(self.lib.ap_cnn_train_step(
                    N._ptr(self.params), N._ptr(self.params_bf16), N._ptr(grads), N._ptr(m1), N._ptr(m2), N._ptr(xb),
                    N._ptr(tb), batch, ctypes.c_float(lr_t), step, ctypes.c_float(weight_decay), N._ptr(loss_d),
                    N._ptr(ws), ws.numel(), N._stream()), "ap_cnn_train_step")
                if b0 == 0:
                    losses.append(loss_d.clone())
            if log_every and (c + 1) % log_every == 0:
                print(f"chunk {c + 1}/{n_chunks} step {step} loss {losses[-1].item():.4f}", flush=True)
        self.history = [float(v.item()) for v in losses]
        return self.history

    def loss(self, st: StampSet, n: int) -> float:
        """Mean squared standardised error on a stamp set."""
        x, lscale = self.prepare(st.data, st.sigma, n)
        out = self.forward(x, n)
        raw = _targets(torch.tensor(st.truth, device=self.device), lscale)
        t = (raw - self.mean.double()) / self.std.double()
        return float(torch.mean((out[:, :N_OUT].double() - t) ** 2).item())


# ---- fits from the two kinds of initial values --------------------------------------------
def moments_init(st: StampSet, n: int, sky_F: float = 0.0) -> torch.Tensor:
    lib = N.lib()
    dev = st.data.device
    sky = torch.full((n,), 10.0**sky_F, dtype=torch.float32, device=dev)
    skyF = torch.full((n,), sky_F, dtype=torch.float64, device=dev)
    out = torch.empty((n, 8), dtype=torch.float64, device=dev)
    N.check(lib.ap_moments_init(N._ptr(st.data), N._ptr(sky), N._ptr(st.sigma.contiguous()), N._ptr(skyF), n,
                                N._ptr(out), N._stream()), "ap_moments_init")
    return out


def heuristic_init(st: StampSet, n: int, sky_F: float = 0.0) -> torch.Tensor:
    """The reference's own initial values of every stamp (``Model.initialize()``: centre of
    light, angular-centre PA, flattest-isophote q, n / Re / Ie from Nelder-Mead on the binned
    median profile), computed by ``ap_reference_init``; the sky slot holds ``sky_F``."""
    vals = torch.zeros((n, 8), dtype=torch.float64, device=st.data.device)
    vals[:, 7] = sky_F
    out, _ = st.batch.reference_init(st.data, None, vals, 0)
    return out


def _lm(st: StampSet, init: torch.Tensor, lm_options):
    b = st.batch
    rep = N.values_to_rep(init, 0x7F)
    return b.lm_fit(st.data, st.weight, None, st.psf, init.contiguous(), rep, lm_options)


def plain_fit(st: StampSet, n: int, lm_options=None):
    """The plain method: LM from the reference's heuristic initial values."""
    init = heuristic_init(st, n)
    return init, _lm(st, init, lm_options or N.make_lm_options())


def subset(st: StampSet, idx) -> StampSet:
    """The stamps ``idx`` (host indices) of ``st`` as their own StampSet and plan."""
    idx = np.asarray(idx, dtype=np.int64)
    dev = st.data.device
    shapes = st.batch.psf_shapes
    off = np.concatenate([[0], np.cumsum([kx * ky for kx, ky in shapes])])
    b = _stamp_batch([shapes[i] for i in idx], dev)
    pix = torch.as_tensor((idx[:, None] * IMG * IMG + np.arange(IMG * IMG)[None, :]).reshape(-1), device=dev)
    psf_idx = torch.as_tensor(np.concatenate([np.arange(off[i], off[i + 1]) for i in idx]), device=dev)
    t = torch.as_tensor(idx, device=dev)
    return StampSet(st.truth[idx], st.data[pix].contiguous(), st.weight[pix].contiguous(), st.psf[psf_idx].contiguous(),
                    st.sigma[t].contiguous(), b)


def learned_fit(net: InitNet, st: StampSet, n: int, lm_options=None, judge_sigma: float = 5.0):
    """LM from the CNN proposal, or from the moments values where those have the lower chi^2;
    then LM's final chi^2 judges the result: a stamp whose chi^2/ndf ends more than
    ``judge_sigma`` standard deviations (sqrt(2 / ndf)) above 1 is fitted again by the plain
    method (LM from the reference's heuristic initial values) and keeps the better fit.
    Returns (initial values, which [0 proposal, 1 moments, 2 plain refit], LM results)."""
    lib = N.lib()
    b = st.batch
    lmo = lm_options or N.make_lm_options()
    prop = net.propose(st.data, st.sigma, n)
    fall = moments_init(st, n)
    c_p = b.chi2(st.data, st.weight, None, b.render(prop, st.psf))
    c_f = b.chi2(st.data, st.weight, None, b.render(fall, st.psf))
    init = torch.empty_like(prop)
    which = torch.empty(n, dtype=torch.int32, device=prop.device)
    N.check(lib.ap_select_init(N._ptr(prop), N._ptr(fall), N._ptr(c_p), N._ptr(c_f), n, N._ptr(init), N._ptr(which),
                               N._stream()), "ap_select_init")
    state, chi2, iters, status = _lm(st, init, lmo)
    ndf = IMG * IMG - 7  # unmasked pixels - free parameters
    bad = torch.nonzero(chi2 > 1.0 + judge_sigma * math.sqrt(2.0 / ndf)).reshape(-1)
    if bad.numel():
        idx = bad.cpu().numpy()
        sub = subset(st, idx)
        h = heuristic_init(sub, len(idx))
        s2, c2, i2, t2 = _lm(sub, h, lmo)
        better = c2 < chi2[bad]
        keep = bad[better]
        if keep.numel():
            sel = better.nonzero().reshape(-1)
            state[keep] = s2[sel]
            chi2[keep] = c2[sel]
            iters[keep] = iters[keep] + i2[sel]
            status[keep] = t2[sel]
            init[keep] = h[sel]
            which[keep] = 2
    return init, which, (state, chi2, iters, status)


def learned_fit_host(net: InitNet, batches, plan: "N.StampBatch", n: int, lm_options=None,
                     judge_sigma: float = 5.0):
    """:func:`learned_fit` of batch after batch of stamps held in host memory.  ``batches`` yields
    (data, weight, psf, sigma) host tensors (pinned for asynchronous copies) in the layout of
    ``plan`` (``n`` stamps).  Each batch is copied to the device on a copy stream into one of two
    input buffer sets while the previous batch is fitted, so the host-to-device transfer overlaps
    the fit instead of preceding it.  Yields, per batch, (state, chi^2, iterations, status) on the
    host."""
    dev = plan.device
    cur = torch.cuda.current_stream(dev)
    copy = torch.cuda.Stream(device=dev)
    bufs, sets = [None, None], [None, None]
    copied = [torch.cuda.Event(), torch.cuda.Event()]
    used = [torch.cuda.Event(), torch.cuda.Event()]
    it = iter(batches)

    def upload(slot, host):
        if bufs[slot] is None:
            bufs[slot] = [torch.empty(h.shape, dtype=h.dtype, device=dev) for h in host]
            sets[slot] = StampSet(np.zeros((n, 8)), bufs[slot][0], bufs[slot][1], bufs[slot][2], bufs[slot][3], plan)
        copy.wait_event(used[slot])  # the fit that read this set is done with it
        with torch.cuda.stream(copy):
            for d_, h_ in zip(bufs[slot], host):
                d_.copy_(h_, non_blocking=True)
        copied[slot].record(copy)

    nxt = next(it, None)
    if nxt is None:
        return
    upload(0, nxt)
    k = 0
    while nxt is not None:
        slot = k % 2
        nxt = next(it, None)
        if nxt is not None:
            upload(1 - slot, nxt)
        cur.wait_event(copied[slot])
        _, _, (state, chi2, iters, status) = learned_fit(net, sets[slot], n, lm_options, judge_sigma)
        used[slot].record(cur)
        yield state.cpu(), chi2.cpu(), iters.cpu(), status.cpu()
        k += 1
