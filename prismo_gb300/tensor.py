"""Anisotropic (tensor) materials and their field update (materials/tensor.py).

``TensorComponents`` and ``TensorMaterial`` restate the reference's containers
(tensor.py:17-312) on NumPy: the full 3x3 matrix (uniform, or per cell with the
two tensor axes last), the diagonal test, and the inverse tensors the update
uses.  ``AnisotropicUpdater`` (tensor.py:437-590) applies
    E' = E + (dt/eps0) [eps]^-1 curl H,   H' = H - (dt/mu0) [mu]^-1 curl E
to device arrays with the native kernel (csrc/aniso.cu, ``pc_aniso_update``):
division by the diagonal for diagonal tensors, the inverse matrix otherwise,
rounded in the reference's evaluation order (float64 equals the NumPy result
bit for bit).  Inputs are torch tensors or this package's device arrays on the
GPU; the results are new device arrays, as the reference returns new arrays.
"""

from __future__ import annotations

import ctypes as C
from dataclasses import dataclass
from typing import Optional, Union

import numpy as np

from . import _lib

EPS0 = 8.854187817e-12
MU0 = 4 * np.pi * 1e-7

Num = Union[float, np.ndarray]


@dataclass
class TensorComponents:
    """tensor.py:17-108: diagonal, symmetric off-diagonal and (optional)
    asymmetric components, scalars or arrays."""

    xx: Num
    yy: Num
    zz: Num
    xy: Num = 0.0
    xz: Num = 0.0
    yz: Num = 0.0
    yx: Optional[Num] = None
    zx: Optional[Num] = None
    zy: Optional[Num] = None

    def is_diagonal(self) -> bool:
        return bool(np.all(np.asarray(self.xy) == 0) and np.all(np.asarray(self.xz) == 0) and
                    np.all(np.asarray(self.yz) == 0) and
                    all(v is None or np.all(np.asarray(v) == 0) for v in (self.yx, self.zx, self.zy)))

    def is_symmetric(self) -> bool:
        return all(v is None for v in (self.yx, self.zx, self.zy)) or bool(
            np.allclose(self.xy, self.yx if self.yx is not None else self.xy) and
            np.allclose(self.xz, self.zx if self.zx is not None else self.xz) and
            np.allclose(self.yz, self.zy if self.zy is not None else self.yz))

    def to_full_matrix(self) -> np.ndarray:
        """[..., 3, 3]; the lower triangle mirrors the upper one unless given."""
        yx = self.xy if self.yx is None else self.yx
        zx = self.xz if self.zx is None else self.zx
        zy = self.yz if self.zy is None else self.zy
        rows = [[self.xx, self.xy, self.xz], [yx, self.yy, self.yz], [zx, zy, self.zz]]
        shape = np.broadcast_shapes(*(np.shape(v) for r in rows for v in r))
        m = np.zeros(shape + (3, 3))
        for i in range(3):
            for j in range(3):
                m[..., i, j] = rows[i][j]
        return m


class TensorMaterial:
    """tensor.py:110-312: [eps] and [mu] (relative); mu defaults to the identity."""

    def __init__(self, epsilon: TensorComponents, mu: Optional[TensorComponents] = None, name: str = "",
                 backend=None):
        self.epsilon = epsilon
        self.mu = mu if mu is not None else TensorComponents(xx=1.0, yy=1.0, zz=1.0)
        self.name = name or "AnisotropicMaterial"
        self.epsilon_tensor = self.epsilon.to_full_matrix()
        self.mu_tensor = self.mu.to_full_matrix()
        self.is_diagonal = self.epsilon.is_diagonal() and self.mu.is_diagonal()
        self.is_symmetric = self.epsilon.is_symmetric() and self.mu.is_symmetric()

    @staticmethod
    def _inverse(t: np.ndarray, comps: TensorComponents, diagonal: bool) -> np.ndarray:
        if diagonal:
            inv = np.zeros_like(t)
            inv[..., 0, 0] = 1.0 / np.asarray(comps.xx)
            inv[..., 1, 1] = 1.0 / np.asarray(comps.yy)
            inv[..., 2, 2] = 1.0 / np.asarray(comps.zz)
            return inv
        return np.linalg.inv(t)  # batched over leading axes

    def get_inverse_epsilon(self) -> np.ndarray:
        return self._inverse(self.epsilon_tensor, self.epsilon, self.is_diagonal)

    def get_inverse_mu(self) -> np.ndarray:
        return self._inverse(self.mu_tensor, self.mu, self.is_diagonal)


def _torch():
    import torch

    return torch


class AnisotropicUpdater:
    """tensor.py:437-590 on the device.  ``tensor_material``: this module's
    TensorMaterial or the reference's (same attributes)."""

    def __init__(self, tensor_material, dt: float, backend=None):
        self.material = tensor_material
        self.dt = dt
        self.eps0 = EPS0
        self.mu0 = 4 * np.pi * 1e-7
        self.inv_epsilon = tensor_material.get_inverse_epsilon()
        self.inv_mu = tensor_material.get_inverse_mu()
        self.lib = _lib.load()
        self._coef_cache = {}

    def _coefficients(self, kind: str, like):
        """(device per-cell array or None, host uniform list) for the E or H update."""
        torch = _torch()
        diag = bool(self.material.is_diagonal)
        if diag:
            comps = self.material.epsilon if kind == "E" else self.material.mu
            vals = [comps.xx, comps.yy, comps.zz]
        else:
            inv = self.inv_epsilon if kind == "E" else self.inv_mu
            vals = [inv[..., i, j] for i in range(3) for j in range(3)]
        if all(np.ndim(v) == 0 for v in vals):
            return None, [float(v) for v in vals]
        key = (kind, like.dtype, tuple(like.shape))
        if key not in self._coef_cache:
            arr = np.stack([np.broadcast_to(np.asarray(v, dtype=np.float64), tuple(like.shape)) for v in vals])
            self._coef_cache[key] = torch.as_tensor(np.ascontiguousarray(arr), device=like.device).to(like.dtype)
        return self._coef_cache[key], [0.0] * 9

    def _update(self, F, curl, kind: str):
        torch = _torch()
        ts = [getattr(x, "tensor", x) for x in F] + [getattr(x, "tensor", x) for x in curl]
        like = ts[0]
        if like.dtype not in (torch.float32, torch.float64) or not like.is_cuda:
            raise TypeError("AnisotropicUpdater works on float32 or float64 CUDA arrays")
        ts = [t.to(like.dtype).contiguous() for t in ts]
        if any(tuple(t.shape) != tuple(like.shape) for t in ts):
            raise ValueError("fields and curls must have the same shape")
        out = [torch.empty_like(like) for _ in range(3)]
        d_coef, uni = self._coefficients(kind, like)
        diag = bool(self.material.is_diagonal)
        scale = self.dt / (self.eps0 if kind == "E" else self.mu0)
        P = C.c_void_p * 3
        u = (C.c_double * 9)(*(uni + [0.0] * (9 - len(uni))))
        _lib.check(self.lib.pc_aniso_update(
            8 if like.dtype == torch.float64 else 4, 1 if diag else 0, 1 if kind == "E" else -1,
            P(*[t.data_ptr() for t in ts[:3]]), P(*[t.data_ptr() for t in ts[3:]]), P(*[t.data_ptr() for t in out]),
            like.numel(), None if d_coef is None else d_coef.data_ptr(), u, scale,
            C.c_void_p(torch.cuda.current_stream(like.device).cuda_stream)), "pc_aniso_update")
        return tuple(out)

    def update_e_from_curl_h(self, E, curl_H):
        """E' = E + (dt/eps0) [eps]^-1 curl H (tensor.py:482-536)."""
        return self._update(E, curl_H, "E")

    def update_h_from_curl_e(self, H, curl_E):
        """H' = H - (dt/mu0) [mu]^-1 curl E (tensor.py:538-589)."""
        return self._update(H, curl_E, "H")
