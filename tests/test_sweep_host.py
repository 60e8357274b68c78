"""CPU checks of the batched-sweep host logic (prismo_gb300/sweep.py): design
generator, fill-fraction rasterisation, TE0 mode solver, port layout and the
S-parameter definitions."""

import math

import numpy as np
import pytest

from prismo_gb300 import sweep as S


def test_design_generator_ranges_and_determinism():
    ds = [S.coupler_design(s) for s in range(200)]
    assert all(400 <= d.nx <= 1200 and 200 <= d.ny <= 800 for d in ds)
    assert all(0.4e-6 <= d.width <= 0.6e-6 and 0.1e-6 <= d.gap <= 0.4e-6 and 2e-6 <= d.length <= 10e-6 for d in ds)
    assert S.coupler_design(17) == S.coupler_design(17)
    p = S.coupler_design(5).params()
    assert np.all((p >= 0) & (p <= 1))
    d2 = S.design_from_params(p, nx=S.coupler_design(5).nx, ny=S.coupler_design(5).ny)
    assert abs(d2.width - S.coupler_design(5).width) < 1e-15 and abs(d2.length - S.coupler_design(5).length) < 1e-15


def test_fill_fraction_rasterisation():
    d = S.DX
    # a strip covering 2.5 cells in y: two full cells and one half cell
    eps = S.fill_eps(4, 10, [(0.0, 4 * d, 3 * d, 5.5 * d)], d)
    col = eps[1]
    assert np.allclose(col[3:5], S.EPS_SI) and np.allclose(col[[0, 1, 2, 6, 7, 8, 9]], S.EPS_SIO2)
    assert abs(col[5] - (S.EPS_SIO2 + 0.5 * (S.EPS_SI - S.EPS_SIO2))) < 1e-12
    # the permittivity integral equals the strip area (fill fractions add up)
    eps = S.fill_eps(50, 40, [(3.3 * d, 20.7 * d, 5.25 * d, 9.6 * d)], d)
    area = ((eps - S.EPS_SIO2) / (S.EPS_SI - S.EPS_SIO2)).sum() * d * d
    assert abs(area - (17.4 * d) * (4.35 * d)) < 1e-9 * d * d


def test_fill_over_the_strip_band_equals_the_whole_grid_fill():
    """fill_eps accumulates area fractions over the strips' y band only; the
    cladding outside it must come out bit-identical to a fill over the whole grid
    (clad + (core - clad) * 0), and so must the band."""
    d = S.DX
    for seed in (0, 3, 17):
        L = S.coupler_layout(S.coupler_design(seed))
        rects = [(0.0, L.nx * d, L.y_a - L.design.width / 2, L.y_a + L.design.width / 2),
                 (1.3 * d, 40.2 * d, L.y_lead - L.design.width / 2, L.y_lead + L.design.width / 2)]
        full = np.zeros((L.nx, L.ny))
        for x0, x1, y0, y1 in rects:
            full += np.outer(S._overlap(L.nx, d, x0, x1), S._overlap(L.ny, d, y0, y1))
        np.clip(full, 0.0, 1.0, out=full)
        full *= S.EPS_SI - S.EPS_SIO2
        full += S.EPS_SIO2
        assert np.array_equal(S.fill_eps(L.nx, L.ny, rects, d), full)


def test_te0_mode_is_symmetric_and_guided():
    d = S.DX
    ny = 80
    w = 0.5e-6
    eps = S.fill_eps(2, ny, [(0, 2 * d, ny * d / 2 - w / 2, ny * d / 2 + w / 2)], d)
    line = 0.5 * (eps[0, :-1] + eps[0, 1:])
    prof, beta = S.te0_mode(line, d, S.F0, S.sweep_dt())
    k0 = 2 * math.pi * S.F0 / S.C0
    neff = beta / k0
    assert math.sqrt(S.EPS_SIO2) < neff < math.sqrt(S.EPS_SI)
    assert prof.max() == 1.0 and np.all(prof > -1e-9)  # fundamental: no sign change
    np.testing.assert_allclose(prof, prof[::-1], atol=1e-6)  # centred strip
    # dispersion: neff decreases with wavelength (increases with frequency)
    b2 = S.te0_beta(line, d, np.array([S.F0 * 0.95, S.F0 * 1.05]), S.sweep_dt())
    assert b2[1] / (k0 * 1.05) > b2[0] / (k0 * 0.95)


@pytest.mark.parametrize("seed", [0, 7, 33])
def test_coupler_layout_ports_and_domain(seed):
    d = S.coupler_design(seed)
    L = S.coupler_layout(d)
    assert L.nx >= d.nx and L.ny == d.ny and L.eps.shape == (L.nx, L.ny)
    t = S.CPML
    for p in [L.src] + L.ports:
        assert t <= p.x < L.nx - 1 - t
        assert p.y0 >= t and p.y0 + p.n <= L.ny - 1 - t
        assert p.profile.shape == (p.n,) and abs(p.profile.max() - 1.0) < 1e-12
    p1, p2, p3, p4 = L.ports
    assert p1.x == p4.x and p2.x == p3.x and p2.x > p1.x
    assert p2.x < L.nx - t - 1 and (p2.x - p1.x) * S.DX > d.length
    # guide B's leads and guide A are separated: their windows do not overlap
    assert p3.y0 + p3.n <= p2.y0 and p4.y0 + p4.n <= p1.y0
    # normalisation domain: guide A alone, same source and port 1 rows
    assert L.norm_eps.shape == (L.norm_nx, L.ny) and L.norm_nx > p1.x + t


def test_s_parameter_definitions():
    L = S.coupler_layout(S.coupler_design(2))
    rng = np.random.default_rng(0)
    nf = 5
    inc = rng.standard_normal(nf) + 1j * rng.standard_normal(nf)
    norm_spec = np.outer(inc, L.ports[0].profile)  # pure port-1 mode in the normalisation run
    coeff = [0.1 - 0.05j, 0.8 + 0.1j, 0.3j, 0.02]
    spec = [np.outer(inc * c, p.profile) for c, p in zip(coeff, L.ports)]
    spec[0] = spec[0] + norm_spec  # incident + reflected wave at port 1
    Sm = S.s_parameters(spec, norm_spec, L)
    for k in range(4):
        np.testing.assert_allclose(Sm[k], coeff[k], atol=1e-12)
    # de-embedding is a unit-modulus phase that inverts exactly
    f = S.sweep_freqs(nf)
    Sd = S.deembed(Sm, L, f)
    np.testing.assert_allclose(np.abs(Sd), np.abs(Sm), rtol=1e-12)
    np.testing.assert_allclose(S.deembed(Sd, L, f, inverse=True), Sm, atol=1e-12)


def test_instances_pair_coupler_and_normalisation():
    Ls = [S.coupler_layout(S.coupler_design(s)) for s in (1, 2)]
    inst = S.instances_for(Ls)
    assert len(inst) == 4
    assert len(inst[0].ports) == 4 and len(inst[1].ports) == 1
    assert inst[1].ports[0] is Ls[0].ports[0] and inst[1].src is Ls[0].src
