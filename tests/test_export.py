"""Host-side export (prismo_gb300.export): the Touchstone table of
analysis/sparameters.py:233-279 and the Parquet column layout of
io/exporters/parquet_exporter.py:195-251, on CPU."""

import importlib.util
import os
from types import SimpleNamespace

import numpy as np
import pytest

from helpers import SOURCE_TREES
from prismo_gb300 import export as X


def _reference_sparameters():
    for root in SOURCE_TREES:
        p = os.path.join(root, "prismo", "analysis", "sparameters.py") if root else ""
        if p and os.path.exists(p):
            spec = importlib.util.spec_from_file_location("_ref_sparameters", p)
            mod = importlib.util.module_from_spec(spec)
            spec.loader.exec_module(mod)
            return mod
    return None


def test_touchstone_matches_reference_writer(tmp_path):
    rng = np.random.default_rng(0)
    f = np.linspace(180e12, 200e12, 5)
    s = rng.standard_normal((5, 3, 3)) + 1j * rng.standard_normal((5, 3, 3))
    X.export_touchstone(tmp_path / "a.s3p", f, s, comments=["coupler sweep", "design 7"])
    f2, s2 = X.read_touchstone(tmp_path / "a.s3p")
    np.testing.assert_allclose(f2, f, rtol=1e-10)
    np.testing.assert_allclose(s2, s, rtol=1e-9, atol=1e-12)
    ref = _reference_sparameters()
    if ref is None:
        pytest.skip("reference source tree not present")
    ref.export_touchstone(tmp_path / "b.s3p", f, s, comments=["coupler sweep", "design 7"])
    assert (tmp_path / "a.s3p").read_text() == (tmp_path / "b.s3p").read_text()


def test_parquet_sparameters_and_sweep_table(tmp_path):
    pq = pytest.importorskip("pyarrow.parquet")
    f = np.array([1.9e14, 2.0e14])
    sp = {"S21": np.array([0.5 + 0.5j, -0.1j]), "S11": np.array([0.01, 0.02 + 0.01j])}
    p = X.export_sparameters_parquet("dev", f, sp, metadata={"w": 0.5}, output_dir=tmp_path)
    t = pq.read_table(p).to_pydict()
    assert list(t)[:5] == ["frequency_Hz", "S21_magnitude", "S21_phase_deg", "S21_real", "S21_imag"]
    np.testing.assert_allclose(t["S21_magnitude"], np.abs(sp["S21"]))
    np.testing.assert_allclose(t["S11_phase_deg"], np.angle(sp["S11"], deg=True))
    assert (tmp_path / "dev.meta.json").exists()

    designs = [SimpleNamespace(seed=s, nx=400 + s, ny=200 + s, width=0.5e-6, gap=0.2e-6, length=3e-6 + s * 1e-7)
               for s in range(3)]
    S = np.arange(3 * 4 * 2).reshape(3, 4, 2) * (1 + 0.5j)
    res = SimpleNamespace(designs=designs, S=S)
    q = X.export_sweep_parquet(res, f, tmp_path / "sweep.parquet")
    t = pq.read_table(q).to_pydict()
    assert len(t["seed"]) == 6 and t["seed"][:3] == [0, 0, 1]
    np.testing.assert_allclose(t["S31_real"], S[:, 2, :].reshape(-1).real)
    np.testing.assert_allclose(t["S21_imag"], S[:, 1, :].reshape(-1).imag)
    with pytest.raises(ValueError):
        X.export_sweep_parquet(res, f[:1], tmp_path / "bad.parquet")
