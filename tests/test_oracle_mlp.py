"""CPU checks of the float64 surrogate oracle (oracle/mlp64.py) against torch
float64 autograd, and of the surrogate's output representation."""

import numpy as np

from oracle import mlp64

DIMS = (3, 64, 64, 64, 96)


def torch_loss_grads(p, x, t, dims):
    import torch

    pt = torch.tensor(p, dtype=torch.float64, requires_grad=True)
    segs, _ = mlp64.layout(dims)
    a = torch.zeros((x.shape[0], 32), dtype=torch.float64)
    a[:, : x.shape[1]] = torch.tensor(x)
    for l, (w_off, b_off, n, k) in enumerate(segs):
        W = pt[w_off:w_off + n * k].reshape(n, k)
        b = pt[b_off:b_off + n]
        z = a @ W.T + b
        a = torch.nn.functional.silu(z) if l < 3 else z
    loss = torch.mean((a - torch.tensor(t)) ** 2)
    loss.backward()
    return float(loss.detach()), pt.grad.numpy()


def test_oracle_matches_torch_autograd():
    rng = np.random.default_rng(0)
    p = mlp64.init_params(DIMS, rng)
    p += 0.01 * rng.standard_normal(p.shape) * (p != 0)  # nonzero biases stay zero: keep the padding exact
    segs, P = mlp64.layout(DIMS)
    for w_off, b_off, n, k in segs:
        p[b_off:b_off + n] = 0.1 * rng.standard_normal(n)
    x = rng.uniform(-1, 1, size=(48, 3))
    t = rng.standard_normal((48, DIMS[-1]))
    l0, g0 = mlp64.loss_and_grads(p, x, t, DIMS)
    l1, g1 = torch_loss_grads(p, x, t, DIMS)
    assert abs(l0 - l1) <= 1e-12 * abs(l1)
    np.testing.assert_allclose(g0, g1, rtol=1e-9, atol=1e-14)
    # padded input columns of layer 0 have zero gradient
    w_off, _, n, k = segs[0]
    assert np.all(g0[w_off:w_off + n * k].reshape(n, k)[:, 3:] == 0)


def test_oracle_adam_matches_torch():
    import torch

    rng = np.random.default_rng(1)
    p = rng.standard_normal(50)
    m = np.zeros(50)
    v = np.zeros(50)
    pt = torch.tensor(p.copy(), requires_grad=True)
    opt = torch.optim.Adam([pt], lr=1e-2, betas=(0.9, 0.999), eps=1e-8)
    for step in range(1, 6):
        g = rng.standard_normal(50)
        p, m, v = mlp64.adam_step(p, g, m, v, step, 1e-2)
        pt.grad = torch.tensor(g)
        opt.step()
    # torch adds eps outside the bias-corrected sqrt(v); the oracle folds the
    # correction into the step size (as the device kernel does): equal to ~eps
    np.testing.assert_allclose(p, pt.detach().numpy(), rtol=0, atol=1e-5)


def test_surrogate_representation_roundtrip():
    from prismo_gb300 import surrogate as Su
    from prismo_gb300 import sweep as S

    designs = [S.coupler_design(s) for s in range(6)]
    rng = np.random.default_rng(2)
    Sp = rng.standard_normal((6, 4, 64)) + 1j * rng.standard_normal((6, 4, 64))
    v = Su.to_real(Sp)
    assert v.shape == (6, 512)
    np.testing.assert_array_equal(Su.from_real(v), Sp)
    ph = Su.phase_factors(designs)
    np.testing.assert_allclose(np.abs(ph), 1.0, rtol=1e-12)
    # the layout's own port distances
    for d, dist in zip(designs, Su.port_distances([d.length for d in designs])):
        L = S.coupler_layout(d)
        assert abs(dist[1] - L.path) < 1e-12
    x = Su.inputs(designs)
    assert x.shape == (6, 3) and np.all(np.abs(x) <= 1)
    # per-member random Fourier embedding: deterministic, member-specific
    B = Su.rff_matrices()
    e = Su.embed(x, B)
    assert e.shape == (Su.MEMBERS, 6, Su.DIMS[0])
    np.testing.assert_array_equal(e[:, :, :3], np.broadcast_to(x, (Su.MEMBERS, 6, 3)))
    np.testing.assert_array_equal(Su.embed(x, Su.rff_matrices()), e)
    assert not np.allclose(e[0, :, 3:], e[1, :, 3:])
