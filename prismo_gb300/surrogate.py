"""Learned surrogate of the coupler sweep, trained on the device (pc_mlp_* C ABI).

An ensemble of four MLPs 3 -> 256 -> 256 -> 256 -> 512 (SiLU) maps the
normalised geometry (width, gap, coupling length) of a directional coupler
(``prismo_gb300.sweep``) to its S11, S21, S31, S41 spectra at 64 frequencies
(real and imaginary parts: 512 outputs).  Training data come from the batched
FDTD sweep; forward, backward and Adam run in the project's own kernels
(csrc/mlp.cu: bf16 tensor-core GEMMs with float32 accumulation).

Outputs are learned in a de-embedded form, S' = S exp(+i beta_ref(w, f) d(L))
with the TE0 propagation constant of an ideal strip of width w (a fixed table,
interpolated) and the port distances of the layout, which removes the fast
phase exp(-i beta L) that an MLP of three inputs could not follow; predictions
are re-embedded with the same factors, so |S - S_fdtd| = |S' - S'_fdtd| exactly.

The plain FDTD stays the fallback: a design whose ensemble spread (RMS over the
512 outputs of the standard deviation across members) exceeds the gate's
threshold is simulated by the batched FDTD instead.  The threshold is calibrated
(``Ensemble.calibrate``) on designs held out from training whose FDTD spectra are
known: the largest spread at which a stated fraction of the admitted designs lie
within the error bar, so that the gate bounds the predicted error rather than
the raw spread; its thresholds are set per coupling-length band, since the
error depends mainly on the coupling length.
"""

from __future__ import annotations

import ctypes as C
import math
import time
from dataclasses import dataclass
from typing import Sequence

import numpy as np

from . import _lib
from . import sweep as SW

MEMBERS = 4
N_RFF = 14  # random Fourier pairs per member: 3 + 2 x 14 = 31 network inputs
RFF_SIGMA = 2.0
DIMS = (3 + 2 * N_RFF, 256, 256, 256, 512)
THRESHOLD = 1e-3  # S-parameter error bar (RMS over the 512 outputs)
CALIB_QUANTILE = 0.98  # fraction of the calibration designs the gate admits that must be within it
CALIB_SEEDS = range(5000, 6024)  # calibration designs (training: 0-4095, held-out tests: 10000+)
CALIB_BINS = 8  # gate thresholds per coupling-length band (the error's main dependence)
EPOCHS = 2000


# ---------------------------------------------------------------------------
# output representation
# ---------------------------------------------------------------------------
_BETA = {}


def beta_table(nfreq: int = SW.NFREQ, nw: int = 81):
    """beta_ref(w, f): TE0 propagation constant (Yee-discrete) of a strip of width
    w in [0.4, 0.6] um centred on a cell boundary, on a grid of nw widths."""
    key = (nfreq, nw)
    if key not in _BETA:
        freqs = SW.sweep_freqs(nfreq)
        dt = SW.sweep_dt()
        ws = np.linspace(0.4e-6, 0.6e-6, nw)
        tab = np.empty((nw, nfreq))
        for q, w in enumerate(ws):
            half = int(math.ceil((w / 2 + SW.WINDOW_MARGIN) / SW.DX)) + 1
            ny = 2 * half + 2
            yc = (half + 1) * SW.DX
            eps = SW.fill_eps(2, ny, [(0.0, 2 * SW.DX, yc - w / 2, yc + w / 2)], SW.DX)
            line = 0.5 * (eps[0, :-1] + eps[0, 1:])
            tab[q] = SW.te0_beta(line, SW.DX, freqs, dt)
        _BETA[key] = (ws, tab)
    return _BETA[key]


def beta_ref(widths, nfreq: int = SW.NFREQ):
    ws, tab = beta_table(nfreq)
    w = np.clip(np.asarray(widths, dtype=np.float64), ws[0], ws[-1])
    pos = (w - ws[0]) / (ws[1] - ws[0])
    i0 = np.clip(np.floor(pos).astype(int), 0, len(ws) - 2)
    f = (pos - i0)[:, None]
    return tab[i0] * (1 - f) + tab[i0 + 1] * f


def port_distances(lengths) -> np.ndarray:
    """[n][4] reference-plane shifts (m) for S11, S21, S31, S41 (the layout's rules)."""
    L = np.asarray(lengths, dtype=np.float64)
    src_x = SW.CPML + SW.SRC_OFF
    p1 = src_x + SW.PORT_OFF
    xc0 = (p1 + 1 + SW.GAP_IN) * SW.DX
    p2 = np.ceil((xc0 + L) / SW.DX + SW.GAP_IN - 1)
    path = (p2 - p1) * SW.DX
    back = np.full_like(path, 2.0 * (xc0 - (p1 + 1) * SW.DX))
    return np.stack([back, path, path, back], axis=1)


def phase_factors(designs: Sequence[SW.CouplerDesign], nfreq: int = SW.NFREQ) -> np.ndarray:
    """[n][4][nf] exp(+i beta_ref d): multiply S by it to de-embed."""
    beta = beta_ref([d.width for d in designs], nfreq)
    dist = port_distances([d.length for d in designs])
    return np.exp(1j * beta[:, None, :] * dist[:, :, None])


def to_real(Sp: np.ndarray) -> np.ndarray:
    """[n][4][nf] complex -> [n][8 nf] (re, im interleaved per port)."""
    n = Sp.shape[0]
    return np.stack([Sp.real, Sp.imag], axis=2).reshape(n, -1)


def from_real(v: np.ndarray, nfreq: int = SW.NFREQ) -> np.ndarray:
    r = v.reshape(v.shape[0], 4, 2, nfreq)
    return r[:, :, 0, :] + 1j * r[:, :, 1, :]


def inputs(designs: Sequence[SW.CouplerDesign]) -> np.ndarray:
    """[n][3] geometry mapped to [-1, 1]."""
    return np.stack([2.0 * d.params() - 1.0 for d in designs]).astype(np.float32)


def rff_matrices(members: int = MEMBERS, n: int = N_RFF, sigma: float = RFF_SIGMA) -> np.ndarray:
    """Per-member random projections [members][3][n] (fixed seeds: part of the model)."""
    return np.stack([np.random.default_rng(100 + m).normal(0.0, sigma, size=(3, n)) for m in range(members)])


def embed(x: np.ndarray, B: np.ndarray) -> np.ndarray:
    """Network inputs of every member: [members][n][3 + 2 nb] = (x, sin(pi x B_m), cos(pi x B_m)).

    Each member sees the three geometry floats through its own random Fourier
    embedding, so the members interpolate differently between training designs and
    their spread grows where the data leave the map under-determined (the spread
    then tracks the error: the fallback test is meaningful)."""
    x = np.asarray(x, dtype=np.float64)
    z = np.pi * np.einsum("nk,mkj->mnj", x, B)
    xs = np.broadcast_to(x[None], (B.shape[0],) + x.shape)
    return np.concatenate([xs, np.sin(z), np.cos(z)], axis=2).astype(np.float32)


# ---------------------------------------------------------------------------
# the ensemble
# ---------------------------------------------------------------------------
def _init_params(dims, rng):
    """Uniform(+-sqrt(6 / (fan_in + fan_out))) weights, zero biases, zero padding
    columns of layer 0 -- in the device's flat parameter layout."""
    P = 0
    segs = []
    for l in range(4):
        k = 32 if l == 0 else dims[l]
        n = dims[l + 1]
        segs.append((P, P + n * k, n, k))
        P += n * k + n
    p = np.zeros(P, dtype=np.float32)
    for l, (w_off, _, n, k) in enumerate(segs):
        fan_in = dims[l]
        lim = math.sqrt(6.0 / (fan_in + n))
        w = np.zeros((n, k), dtype=np.float32)
        w[:, :fan_in] = rng.uniform(-lim, lim, size=(n, fan_in))
        p[w_off:w_off + n * k] = w.ravel()
    return p


class Ensemble:
    """``members`` MLPs trained side by side by the device kernels (pc_mlp_*)."""

    def __init__(self, members: int = MEMBERS, dims=DIMS, max_batch: int = 8192, seed: int = 0, device=None):
        import torch

        self.torch = torch
        self.lib = _lib.load()
        self.members = int(members)
        self.dims = tuple(int(d) for d in dims)
        self.max_batch = int(max_batch)
        self.device = torch.device(device or "cuda")
        if self.device.type != "cuda":
            raise RuntimeError("the surrogate trains on a CUDA device only")
        d = (C.c_int32 * 5)(*self.dims)
        h = C.c_void_p()
        with torch.cuda.device(self.device):
            _lib.check(self.lib.pc_mlp_create(self.members, self.max_batch, d, C.byref(h)), "pc_mlp_create")
        self.h = h
        self.P = int(self.lib.pc_mlp_param_count(h))
        rng = np.random.default_rng(seed)
        self.set_params(np.stack([_init_params(self.dims, rng) for _ in range(self.members)]))
        nrff = (self.dims[0] - 3) // 2
        self.B = rff_matrices(self.members, nrff) if nrff > 0 else None
        self.x_mean = None
        self.y_mean = self.y_std = None
        self._loss = torch.zeros(self.members, dtype=torch.float32, device=self.device)

    def layout(self):
        out = []
        for l in range(4):
            o = (C.c_int64 * 4)()
            _lib.check(self.lib.pc_mlp_param_layout(self.h, l, o), "pc_mlp_param_layout")
            out.append(tuple(int(v) for v in o))
        return out

    def set_params(self, p: np.ndarray):
        a = np.ascontiguousarray(p, dtype=np.float32).reshape(self.members, self.P)
        _lib.check(self.lib.pc_mlp_set_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float))), "pc_mlp_set_params")

    def params(self) -> np.ndarray:
        a = np.empty((self.members, self.P), dtype=np.float32)
        _lib.check(self.lib.pc_mlp_get_params(self.h, a.ctypes.data_as(C.POINTER(C.c_float))), "pc_mlp_get_params")
        return a

    def grads(self) -> np.ndarray:
        a = np.empty((self.members, self.P), dtype=np.float32)
        _lib.check(self.lib.pc_mlp_get_grads(self.h, a.ctypes.data_as(C.POINTER(C.c_float))), "pc_mlp_get_grads")
        return a

    @property
    def launches(self) -> int:
        return int(self.lib.pc_mlp_launch_count(self.h))

    def set_tensor_path(self, tcgen05):
        """Products on tcgen05 wherever the shape fits (True), on mma.sync (False),
        or chosen by launch size ("auto", the default)."""
        mode = 2 if tcgen05 == "auto" else (1 if tcgen05 else 0)
        _lib.check(self.lib.pc_mlp_set_tensor_path(self.h, mode), "pc_mlp_set_tensor_path")

    def status(self) -> int:
        v = C.c_uint32(0)
        _lib.check(self.lib.pc_mlp_status(self.h, C.byref(v), self._stream()), "pc_mlp_status")
        return int(v.value)

    def _stream(self):
        return self.torch.cuda.current_stream(self.device).cuda_stream

    # -- raw device calls ---------------------------------------------------------
    def forward_raw(self, x):
        """x: device float32 [members][B][din] -> [members][B][dout]."""
        torch = self.torch
        x = x.contiguous()
        B = x.shape[1]
        y = torch.empty((self.members, B, self.dims[-1]), dtype=torch.float32, device=self.device)
        _lib.check(self.lib.pc_mlp_forward(self.h, x.data_ptr(), B, y.data_ptr(), self._stream()), "pc_mlp_forward")
        return y

    def gradients_raw(self, x, t):
        x, t = x.contiguous(), t.contiguous()
        _lib.check(self.lib.pc_mlp_gradients(self.h, x.data_ptr(), t.data_ptr(), x.shape[1], self._loss.data_ptr(),
                                             self._stream()), "pc_mlp_gradients")
        return self._loss

    def train_step_raw(self, x, t, lr, b1=0.9, b2=0.999, eps=1e-8):
        _lib.check(self.lib.pc_mlp_train_step(self.h, x.data_ptr(), t.data_ptr(), x.shape[1], float(lr), b1, b2, eps,
                                              self._loss.data_ptr(), self._stream()), "pc_mlp_train_step")
        return self._loss

    # -- training on S-parameters -----------------------------------------------------
    def fit(self, designs: Sequence[SW.CouplerDesign], S: np.ndarray, epochs: int = 2000, batch: int = 256,
            lr: float = 2e-3, lr_min: float = 2e-5, seed: int = 1, log_every: int = 0):
        """Train every member on (designs, S) with its own shuffles; cosine decay."""
        torch = self.torch
        X = self._features(inputs(designs))
        Y = to_real(S * phase_factors(designs, S.shape[-1]))
        # one scale for every output: the loss then weighs the outputs as the
        # S-parameter error does (a per-output scale would spend the network on
        # the near-constant small outputs)
        self.y_mean = Y.mean(axis=0)
        self.y_std = np.full(Y.shape[1], max(float(Y.std()), 1e-6))
        Yn = ((Y - self.y_mean) / self.y_std).astype(np.float32)
        dev = self.device
        Xd = torch.as_tensor(X, device=dev)
        Yd = torch.as_tensor(Yn, device=dev)
        n = X.shape[1]
        batch = min(batch, (n // 32) * 32)
        mem = torch.arange(self.members, device=dev)[:, None]
        steps_per_epoch = n // batch
        total = epochs * steps_per_epoch
        gen = torch.Generator(device=dev)
        gen.manual_seed(seed)
        history = []
        t0 = time.perf_counter()
        step = 0
        for ep in range(epochs):
            perms = torch.stack([torch.randperm(n, device=dev, generator=gen) for _ in range(self.members)])
            for s in range(steps_per_epoch):
                idx = perms[:, s * batch:(s + 1) * batch]
                lr_s = lr_min + 0.5 * (lr - lr_min) * (1 + math.cos(math.pi * step / total))
                loss = self.train_step_raw(Xd[mem, idx], Yd[idx], lr_s)
                step += 1
            if log_every and (ep % log_every == 0 or ep == epochs - 1):
                history.append((ep, loss.cpu().numpy().copy()))
        torch.cuda.synchronize(dev)
        self.train_seconds = time.perf_counter() - t0
        self.train_steps = step
        return history

    def _features(self, x: np.ndarray) -> np.ndarray:
        """[members][n][din] network inputs for geometry x [n][3]."""
        if self.B is None:
            return np.ascontiguousarray(np.broadcast_to(x[None], (self.members,) + x.shape), dtype=np.float32)
        return embed(x, self.B)

    def predict(self, designs: Sequence[SW.CouplerDesign], nfreq: int = SW.NFREQ, members: bool = False):
        """Ensemble mean S [n][4][nf], spread [n] and (``members``) per-member S
        [members][n][4][nf] (None otherwise)."""
        torch = self.torch
        X = self._features(inputs(designs))
        n = X.shape[1]
        outs = []
        for q in range(0, n, self.max_batch):
            xb = torch.as_tensor(np.ascontiguousarray(X[:, q:q + self.max_batch]), device=self.device)
            outs.append(self.forward_raw(xb))
        y = torch.cat(outs, dim=1).cpu().numpy().astype(np.float64)
        y = y * self.y_std + self.y_mean
        spread = np.sqrt(np.mean(np.var(y, axis=0), axis=1))
        mean = y.mean(axis=0)
        ph = phase_factors(designs, nfreq)
        S = from_real(mean, nfreq) / ph
        S_m = np.stack([from_real(y[m], nfreq) / ph for m in range(self.members)]) if members else None
        return S, spread, S_m

    def calibrate(self, designs: Sequence[SW.CouplerDesign], S_ref: np.ndarray, target: float = THRESHOLD,
                  quantile: float = CALIB_QUANTILE, bins: int = CALIB_BINS) -> np.ndarray:
        """Set the gate from designs held out from training with known FDTD
        S-parameters, one threshold per coupling-length band: admitting the band's
        designs in order of increasing spread, the largest spread at which at least
        ``quantile`` of the admitted designs lie within ``target`` (0 admits none).
        Returns the per-band thresholds."""
        S, spread, _ = self.predict(designs)
        err = s_error(S, S_ref)
        band = self._band(designs, bins)
        thr = np.zeros(bins)
        admitted = np.zeros(bins, dtype=int)
        for b in range(bins):
            sel = np.nonzero(band == b)[0]
            order = sel[np.argsort(spread[sel], kind="stable")]
            ok = err[order] <= target
            frac = np.cumsum(ok) / np.arange(1, len(ok) + 1)
            good = np.nonzero(frac >= quantile)[0]
            if len(good):
                thr[b] = spread[order][good[-1]]
                admitted[b] = good[-1] + 1
        self.thresholds = thr
        self.calibration = {"designs": len(designs), "target": target, "quantile": quantile, "bands": bins,
                            "admitted": admitted.tolist(), "thresholds": thr.tolist()}
        return thr

    @staticmethod
    def _band(designs: Sequence[SW.CouplerDesign], bins: int) -> np.ndarray:
        L = np.array([d.params()[2] for d in designs])
        return np.clip((L * bins).astype(int), 0, bins - 1)

    def gate(self, designs: Sequence[SW.CouplerDesign], spread: np.ndarray, threshold=None) -> np.ndarray:
        """Which designs the ensemble answers: spread under the calibrated band
        threshold (or under ``threshold`` / ``THRESHOLD`` without a calibration)."""
        thr = getattr(self, "thresholds", None)
        if threshold is not None or thr is None:
            return spread <= (THRESHOLD if threshold is None else threshold)
        return spread <= thr[self._band(designs, len(thr))]

    def close(self):
        if getattr(self, "h", None):
            self.lib.pc_mlp_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass


# ---------------------------------------------------------------------------
# surrogate with FDTD fallback
# ---------------------------------------------------------------------------
@dataclass
class PipelineResult:
    S: np.ndarray
    accepted: np.ndarray  # bool [n]
    spread: np.ndarray
    seconds: float
    infer_seconds: float
    fdtd_seconds: float

    @property
    def designs_per_s(self) -> float:
        return len(self.S) / self.seconds


def s_error(S_a: np.ndarray, S_b: np.ndarray) -> np.ndarray:
    """Per design RMS over the 512 real outputs of the difference."""
    d = to_real(S_a - S_b)
    return np.sqrt(np.mean(d * d, axis=1))


def run_pipeline(model: Ensemble, designs: Sequence[SW.CouplerDesign], threshold=None,
                 nsteps: int = SW.STEPS, device=None) -> PipelineResult:
    """Surrogate answers where the ensemble agrees; batched FDTD elsewhere.  The
    gate is the model's calibrated one (``Ensemble.calibrate``), else a spread
    threshold (``threshold`` or ``THRESHOLD``)."""
    torch = model.torch
    torch.cuda.synchronize(model.device)
    t0 = time.perf_counter()
    S, spread, _ = model.predict(designs)
    acc = model.gate(designs, spread, threshold)
    t1 = time.perf_counter()
    fb = [d for d, a in zip(designs, acc) if not a]
    t_fdtd = 0.0
    if fb:
        r = SW.batched_sweep(fb, nsteps=nsteps, device=device)
        t_fdtd = r.seconds
        S = S.copy()
        S[~acc] = r.S
    t2 = time.perf_counter()
    return PipelineResult(S, acc, spread, t2 - t0, t1 - t0, t_fdtd)
