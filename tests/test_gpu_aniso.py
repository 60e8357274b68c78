"""AnisotropicUpdater on the device (csrc/aniso.cu) against the reference's array
expressions (materials/tensor.py:482-589) evaluated with NumPy: float64 equal
bit for bit, float32 within 2e-6 relative (the reference promotes the full-tensor
path to float64)."""

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def reference_update(mat, inv_eps, inv_mu, dt, E, curl_H, H, curl_E):
    """tensor.py:482-589 verbatim in NumPy (the expressions, restated)."""
    eps0, mu0 = 8.854187817e-12, 4 * np.pi * 1e-7
    if mat.is_diagonal:
        e = [E[0] + (dt / eps0) * curl_H[0] / mat.epsilon.xx, E[1] + (dt / eps0) * curl_H[1] / mat.epsilon.yy,
             E[2] + (dt / eps0) * curl_H[2] / mat.epsilon.zz]
        h = [H[0] - (dt / mu0) * curl_E[0] / mat.mu.xx, H[1] - (dt / mu0) * curl_E[1] / mat.mu.yy,
             H[2] - (dt / mu0) * curl_E[2] / mat.mu.zz]
    else:
        e = [E[r] + (dt / eps0) * (inv_eps[..., r, 0] * curl_H[0] + inv_eps[..., r, 1] * curl_H[1] +
                                   inv_eps[..., r, 2] * curl_H[2]) for r in range(3)]
        h = [H[r] + -(dt / mu0) * (inv_mu[..., r, 0] * curl_E[0] + inv_mu[..., r, 1] * curl_E[1] +
                                   inv_mu[..., r, 2] * curl_E[2]) for r in range(3)]
    return e, h


def materials(shape, rng):
    from prismo_gb300.tensor import TensorComponents, TensorMaterial

    u = rng.uniform
    yield TensorMaterial(TensorComponents(xx=2.1, yy=2.3, zz=4.6), TensorComponents(xx=1.0, yy=1.2, zz=0.9))
    yield TensorMaterial(TensorComponents(xx=u(1, 4, shape), yy=u(1, 4, shape), zz=u(1, 4, shape)))
    yield TensorMaterial(TensorComponents(xx=2.2, yy=2.5, zz=3.1, xy=0.3, xz=-0.2, yz=0.1),
                         TensorComponents(xx=1.0, yy=1.1, zz=1.0, xy=0.05))
    yield TensorMaterial(TensorComponents(xx=u(2, 4, shape), yy=u(2, 4, shape), zz=u(2, 4, shape),
                                          xy=u(-0.3, 0.3, shape), xz=u(-0.3, 0.3, shape), yz=u(-0.3, 0.3, shape),
                                          yx=u(-0.3, 0.3, shape)))


@pytest.mark.parametrize("dtype", ["float64", "float32"])
def test_anisotropic_updater_matches_reference_expressions(torch, dtype):
    from prismo_gb300.tensor import AnisotropicUpdater

    rng = np.random.default_rng(11)
    shape = (17, 13, 11)
    dt = 3.3e-17
    for mat in materials(shape, rng):
        arrs = [rng.standard_normal(shape).astype(dtype) for _ in range(12)]
        E, cH, H, cE = arrs[0:3], arrs[3:6], arrs[6:9], arrs[9:12]
        up = AnisotropicUpdater(mat, dt)
        dev = lambda xs: [torch.as_tensor(x, device="cuda") for x in xs]  # noqa: E731
        e = [x.cpu().numpy() for x in up.update_e_from_curl_h(dev(E), dev(cH))]
        h = [x.cpu().numpy() for x in up.update_h_from_curl_e(dev(H), dev(cE))]
        if dtype == "float64":
            we, wh = reference_update(mat, up.inv_epsilon, up.inv_mu, dt, E, cH, H, cE)
            for a, b in zip(e + h, we + wh):
                np.testing.assert_array_equal(a, b)
        else:
            E64, cH64, H64, cE64 = ([x.astype(np.float64) for x in g] for g in (E, cH, H, cE))
            we, wh = reference_update(mat, up.inv_epsilon, up.inv_mu, dt, E64, cH64, H64, cE64)
            for a, b in zip(e + h, we + wh):
                assert np.abs(a - b).max() <= 2e-6 * np.abs(b).max()
