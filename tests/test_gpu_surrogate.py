"""Surrogate kernels (pc_mlp_*) against the float64 oracle (oracle/mlp64.py).

The device computes with bf16 operands and float32 accumulation, so it is
compared with the oracle evaluated on the same bf16-rounded parameters and
inputs; the remaining differences come from bf16 rounding of activations and
back-propagated gradients (about 2^-9 relative each):
  forward output rel L2 <= 1e-2, per-layer gradient rel L2 <= 3e-2,
  one Adam step: |w_dev - w_oracle(g_dev)| <= 1e-6 + 1e-5 |w|.
Members are independent (each one checked against its own oracle).
"""

import numpy as np
import pytest

from oracle import mlp64
from prismo_gb300 import _lib

pytestmark = pytest.mark.gpu

DIMS = (3, 256, 256, 256, 512)


@pytest.fixture(scope="module")
def torch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def bf16_round(a):
    import torch

    return torch.tensor(np.asarray(a, dtype=np.float32)).to(torch.bfloat16).to(torch.float32).numpy().astype(np.float64)


def rel(a, b):
    return np.linalg.norm(a - b) / max(np.linalg.norm(b), 1e-300)


def make(torch, members=2, batch=64, seed=0):
    from prismo_gb300.surrogate import Ensemble

    E = Ensemble(members=members, dims=DIMS, max_batch=batch, seed=seed)
    rng = np.random.default_rng(seed)
    p = E.params().astype(np.float64)
    segs, _ = mlp64.layout(DIMS)
    for m in range(members):
        for w_off, b_off, n, k in segs:
            p[m, b_off:b_off + n] = 0.05 * rng.standard_normal(n)
    p = bf16_round(p)  # the device's bf16 weight copies then equal the masters
    E.set_params(p)
    x = bf16_round(rng.uniform(-1, 1, size=(members, batch, 3)))
    t = rng.standard_normal((members, batch, DIMS[-1]))
    return E, p, x, t


def test_forward_matches_oracle(torch):
    E, p, x, t = make(torch)
    y = E.forward_raw(torch.tensor(x, dtype=torch.float32, device="cuda")).cpu().numpy()
    for m in range(E.members):
        want, _ = mlp64.forward(p[m], x[m], DIMS)
        assert rel(y[m], want) <= 1e-2, rel(y[m], want)
    # a partial batch (rows < max_batch) gives the same rows
    y2 = E.forward_raw(torch.tensor(x[:, :20], dtype=torch.float32, device="cuda")).cpu().numpy()
    np.testing.assert_array_equal(y2, y[:, :20])
    E.close()


def test_gradients_match_oracle(torch):
    E, p, x, t = make(torch, seed=3)
    loss = E.gradients_raw(torch.tensor(x, dtype=torch.float32, device="cuda"),
                           torch.tensor(t, dtype=torch.float32, device="cuda")).cpu().numpy()
    g = E.grads()
    segs, _ = mlp64.layout(DIMS)
    for m in range(E.members):
        l_o, g_o = mlp64.loss_and_grads(p[m], x[m], t[m], DIMS)
        assert abs(loss[m] - l_o) <= 1e-3 * l_o, (loss[m], l_o)
        for l, (w_off, b_off, n, k) in enumerate(segs):
            gw, gw_o = g[m, w_off:w_off + n * k], g_o[w_off:w_off + n * k]
            gb, gb_o = g[m, b_off:b_off + n], g_o[b_off:b_off + n]
            assert rel(gw, gw_o) <= 3e-2, (m, l, "W", rel(gw, gw_o))
            assert rel(gb, gb_o) <= 3e-2, (m, l, "b", rel(gb, gb_o))
        w_off, _, n, k = segs[0]
        assert np.all(g[m, w_off:w_off + n * k].reshape(n, k)[:, 3:] == 0)
    E.close()


def test_adam_step_and_training_progress(torch):
    E, p, x, t = make(torch, seed=5)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    td = torch.tensor(t, dtype=torch.float32, device="cuda")
    E.gradients_raw(xd, td)
    g = E.grads().astype(np.float64)
    E.set_params(p)  # reset Adam
    E.train_step_raw(xd, td, 1e-3)
    got = E.params()
    for m in range(E.members):
        want, _, _ = mlp64.adam_step(p[m], g[m], np.zeros_like(p[m]), np.zeros_like(p[m]), 1, 1e-3)
        np.testing.assert_allclose(got[m], want, rtol=1e-5, atol=1e-6)
    # fit a smooth target: the loss falls by 10x in 300 steps on every member
    rng = np.random.default_rng(7)
    xs = rng.uniform(-1, 1, size=(E.members, 64, 3))
    w = rng.standard_normal((3, DIMS[-1]))
    ts = np.sin(xs @ w)
    xd = torch.tensor(xs, dtype=torch.float32, device="cuda")
    td = torch.tensor(ts, dtype=torch.float32, device="cuda")
    first = E.gradients_raw(xd, td).cpu().numpy().copy()
    for _ in range(300):
        last = E.train_step_raw(xd, td, 2e-3)
    last = E.gradients_raw(xd, td).cpu().numpy()
    assert np.all(last < 0.1 * first), (first, last)
    E.close()


def test_surrogate_gain_over_fdtd_alone(torch):
    """What the trained network adds to the batched FDTD: trained on the batched
    FDTD's spectra of designs 0-4095, its gate calibrated on designs 5000-6023
    (per coupling-length band, the largest ensemble spread at which 98 % of the
    admitted designs are within the 1e-3 error bar), on 128 held-out couplers the pipeline (ensemble answers
    where the spread is under the gate, batched FDTD elsewhere) returns every
    design faster than the batched FDTD alone, at least 95 % of the answered
    designs within an RMS S-parameter error of 1e-3, and the fallback designs
    exactly as the FDTD computes them.  (bench.py --workload surrogate runs the
    256-design held-out set and the 8192-query inference batch.)"""
    from prismo_gb300 import surrogate as Su
    from prismo_gb300 import sweep as S

    train = [S.coupler_design(s) for s in range(4096)]
    calib = [S.coupler_design(s) for s in Su.CALIB_SEEDS]
    test = [S.coupler_design(s) for s in range(10000, 10128)]
    Str = np.concatenate([S.batched_sweep(train[q:q + 1024]).S for q in range(0, 4096, 1024)])
    ref = S.batched_sweep(test)  # the method without the network
    E = Su.Ensemble(max_batch=1024)
    E.fit(train, Str, epochs=Su.EPOCHS)
    E.calibrate(calib, np.concatenate([S.batched_sweep(calib[q:q + 512]).S for q in range(0, len(calib), 512)]))
    res = Su.run_pipeline(E, test)
    err = Su.s_error(res.S, ref.S)
    acc = res.accepted
    within = float(np.mean(err[acc] <= 1e-3)) if acc.any() else 0.0
    print(f"gate {E.calibration}; accepted {acc.sum()}/{len(test)}, within 1e-3 {within:.3f}, "
          f"answered err median {np.median(err[acc]):.2e} max {err[acc].max():.2e}; "
          f"pipeline {res.seconds:.2f} s vs FDTD {ref.seconds:.2f} s")
    assert acc.sum() >= 5
    assert np.all(err[~acc] == 0.0)
    assert within >= 0.95, within
    assert res.seconds < ref.seconds
    E.close()


def test_tcgen05_forward_matches_mma_sync(torch):
    """The forward products on tcgen05 (tensor-memory accumulator) equal the
    mma.sync products up to float32 summation order (rel 1e-5), including a
    partial 128-row tile; the oracle check of the gradients holds on this path."""
    E, p, x, t = make(torch, members=2, batch=320, seed=9)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    E.set_tensor_path(False)
    y0 = E.forward_raw(xd).cpu().numpy()
    E.set_tensor_path(True)
    y1 = E.forward_raw(xd).cpu().numpy()
    assert E.status() == 0
    assert rel(y1, y0) <= 1e-5, rel(y1, y0)
    # an output buffer 4 bytes off 16-byte alignment takes the mma.sync path
    buf = torch.empty(y1.size + 1, dtype=torch.float32, device="cuda")
    _lib.check(E.lib.pc_mlp_forward(E.h, xd.data_ptr(), x.shape[1], buf[1:].data_ptr(), E._stream()),
               "pc_mlp_forward")
    assert rel(buf[1:].cpu().numpy().reshape(y1.shape), y0) <= 1e-6
    for m in range(E.members):
        want, _ = mlp64.forward(p[m], x[m], DIMS)
        assert rel(y1[m], want) <= 1e-2
    E.close()


def test_tcgen05_backward_matches_mma_sync(torch):
    """The data- and weight-gradient products on tcgen05 against the mma.sync
    products: the last layer's weight gradient (the first product, from the same
    bf16 loss gradient) to float32 summation order (rel 1e-5); the layers below
    through bf16-rounded data gradients, where an element can round the other
    way (rel 1e-2); batch 320 leaves a partial 128-row tile."""
    E, p, x, t = make(torch, members=2, batch=320, seed=11)
    xd = torch.tensor(x, dtype=torch.float32, device="cuda")
    td = torch.tensor(t, dtype=torch.float32, device="cuda")
    segs, _ = mlp64.layout(DIMS)
    out = []
    for tc in (False, True):
        E.set_tensor_path(tc)
        E.forward_raw(xd)
        E.gradients_raw(xd, td)
        out.append(E.grads())
    assert E.status() == 0
    g0, g1 = out
    for m in range(E.members):
        for l, (w_off, b_off, n, k) in enumerate(segs):
            a, b = g1[m, w_off:w_off + n * k], g0[m, w_off:w_off + n * k]
            assert rel(a, b) <= (1e-5 if l == 3 else 1e-2), (m, l, rel(a, b))
        l_o, g_o = mlp64.loss_and_grads(p[m], x[m], t[m], DIMS)
        for l, (w_off, b_off, n, k) in enumerate(segs):
            assert rel(g1[m, w_off:w_off + n * k], g_o[w_off:w_off + n * k]) <= 3e-2, (m, l)
    E.close()
