"""Export of S-parameters and sweep results (host only).

``export_touchstone`` writes the Touchstone table of analysis/sparameters.py:233-279
(same header, option line and row layout: a wire format has to match);
``export_sparameters_parquet`` writes the column layout of
io/exporters/parquet_exporter.py:195-251 (frequency_Hz, then per parameter
magnitude, phase in degrees, real and imaginary parts, and an optional
.meta.json) through pyarrow, since the reference's polars is not a dependency
here.  ``export_sweep_parquet`` flattens a batched sweep (sweep.SweepResult) into
one row per design and frequency: the wire format for sweep outputs.
"""

from __future__ import annotations

import json
from pathlib import Path
from typing import Optional, Sequence

import numpy as np


def export_touchstone(filename, frequencies, s_matrix, z0: float = 50.0, comments: Optional[Sequence[str]] = None):
    """S-matrix [n_freq][n_ports][n_ports] to a .sNp file, real/imaginary pairs in
    row-major port order."""
    s_matrix = np.asarray(s_matrix)
    n = s_matrix.shape[1]
    lines = ["! Touchstone file generated by Prismo"]
    lines += [f"! {c}" for c in (comments or [])]
    lines.append(f"# Hz S RI R {z0}")
    for fi, f in enumerate(np.asarray(frequencies)):
        row = [f"{f:.10e}"]
        for i in range(n):
            for j in range(n):
                v = s_matrix[fi, i, j]
                row.append(f"{v.real:.10e} {v.imag:.10e}")
        lines.append(" ".join(row))
    with open(filename, "w") as fh:
        fh.write("\n".join(lines) + "\n")


def read_touchstone(filename):
    """(frequencies, S [n_freq][n][n]) of a file written by export_touchstone."""
    rows = [ln.split() for ln in open(filename) if ln.strip() and not ln.startswith(("!", "#"))]
    a = np.array(rows, dtype=np.float64)
    n = int(round(np.sqrt((a.shape[1] - 1) / 2)))
    s = (a[:, 1::2] + 1j * a[:, 2::2]).reshape(-1, n, n)
    return a[:, 0], s


def _write_parquet(path: Path, columns: dict, compression: str):
    try:
        import pyarrow as pa
        import pyarrow.parquet as pq
    except ImportError as e:  # pragma: no cover - depends on the environment
        raise ImportError("pyarrow is required for Parquet export") from e
    pq.write_table(pa.table({k: np.asarray(v) for k, v in columns.items()}), str(path), compression=compression)


def export_sparameters_parquet(filename, frequencies, sparameters: dict, metadata: Optional[dict] = None,
                               output_dir=".", compression: str = "snappy") -> Path:
    """parquet_exporter.py:195-251 layout; returns the file's path."""
    out = Path(output_dir) / f"{filename}.parquet"
    cols = {"frequency_Hz": np.asarray(frequencies, dtype=np.float64)}
    for name, v in sparameters.items():
        v = np.asarray(v)
        cols[f"{name}_magnitude"] = np.abs(v)
        cols[f"{name}_phase_deg"] = np.angle(v, deg=True)
        cols[f"{name}_real"] = np.real(v)
        cols[f"{name}_imag"] = np.imag(v)
    _write_parquet(out, cols, compression)
    if metadata:
        with open(out.with_suffix(".meta.json"), "w") as fh:
            json.dump(metadata, fh, indent=2)
    return out


def export_sweep_parquet(result, frequencies, path, compression: str = "snappy") -> Path:
    """One row per (design, frequency) of a batched sweep: design seed, grid size,
    width / gap / length (m), frequency, and S11, S21, S31, S41 as real and
    imaginary columns."""
    S = np.asarray(result.S)
    nd, nport, nf = S.shape
    freqs = np.asarray(frequencies, dtype=np.float64)
    if freqs.size != nf:
        raise ValueError("frequencies do not match the result's spectra")
    rep = lambda x: np.repeat(np.asarray(x), nf)  # noqa: E731
    d = result.designs
    cols = {"seed": rep([x.seed for x in d]), "nx": rep([x.nx for x in d]), "ny": rep([x.ny for x in d]),
            "width_m": rep([x.width for x in d]), "gap_m": rep([x.gap for x in d]),
            "length_m": rep([x.length for x in d]), "frequency_Hz": np.tile(freqs, nd)}
    for k in range(nport):
        v = S[:, k, :].reshape(-1)
        cols[f"S{k + 1}1_real"] = v.real
        cols[f"S{k + 1}1_imag"] = v.imag
    out = Path(path)
    _write_parquet(out, cols, compression)
    return out
