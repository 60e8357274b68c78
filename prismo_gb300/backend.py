"""The "cuda" backend: Prismo's array-provider interface (backends/base.py:14-219)
on device memory, plus the backend registry (backends/backend_manager.py).

Arrays are ``DeviceArray`` objects that hold (or resolve to) a CUDA tensor; every
operation stays on the device.  ``__array__`` is the one explicit device-to-host
copy, for user code that hands a field to NumPy.
"""

from __future__ import annotations

import math
import warnings
from abc import ABC, abstractmethod
from typing import Optional

import numpy as np


def _torch():
    import torch

    return torch


_NP_TO_TORCH = None


def _dtype_to_torch(dtype):
    torch = _torch()
    global _NP_TO_TORCH
    if _NP_TO_TORCH is None:
        _NP_TO_TORCH = {
            np.dtype(np.float32): torch.float32, np.dtype(np.float64): torch.float64,
            np.dtype(np.complex64): torch.complex64, np.dtype(np.complex128): torch.complex128,
            np.dtype(np.int32): torch.int32, np.dtype(np.int64): torch.int64, np.dtype(np.bool_): torch.bool,
        }
    if dtype is None:
        return None
    if isinstance(dtype, torch.dtype):
        return dtype
    return _NP_TO_TORCH[np.dtype(dtype)]


def _to_index(idx, device):
    """NumPy-style index (ints, slices, np.ix_ arrays, masks) -> torch index."""
    torch = _torch()
    if isinstance(idx, tuple):
        return tuple(_to_index(i, device) for i in idx)
    if isinstance(idx, DeviceArray):
        return idx.tensor
    if isinstance(idx, np.ndarray):
        return torch.as_tensor(idx, device=device)
    if isinstance(idx, (list, range)):
        return torch.as_tensor(np.asarray(idx), device=device)
    return idx


def _is_basic(idx) -> bool:
    items = idx if isinstance(idx, tuple) else (idx,)
    return all(isinstance(i, (int, slice, type(None), type(Ellipsis))) for i in items)


class DeviceArray:
    """NumPy-flavoured handle on a CUDA tensor (or on a view that follows a field
    buffer across ping-pong swaps, when built from a resolver)."""

    __array_priority__ = 1000

    def __init__(self, tensor=None, resolver=None):
        if (tensor is None) == (resolver is None):
            raise ValueError("give exactly one of tensor / resolver")
        self._tensor = tensor
        self._resolver = resolver

    # -- core --------------------------------------------------------------
    @property
    def tensor(self):
        return self._tensor if self._resolver is None else self._resolver()

    @property
    def shape(self):
        return tuple(self.tensor.shape)

    @property
    def ndim(self):
        return self.tensor.dim()

    @property
    def size(self):
        return int(self.tensor.numel())

    @property
    def dtype(self):
        return np.dtype(str(self.tensor.dtype).replace("torch.", ""))

    @property
    def nbytes(self):
        t = self.tensor
        return int(t.numel() * t.element_size())

    @property
    def device(self):
        return self.tensor.device

    def __len__(self):
        return self.shape[0]

    def __repr__(self):
        return f"DeviceArray(shape={self.shape}, dtype={self.dtype}, device={self.device})"

    # -- conversion ----------------------------------------------------------
    def to_numpy(self) -> np.ndarray:
        return self.tensor.detach().cpu().numpy()

    def __array__(self, dtype=None, copy=None):
        a = self.to_numpy()
        return a.astype(dtype) if dtype is not None else a

    def copy(self):
        return DeviceArray(self.tensor.clone())

    def fill(self, value):
        self.tensor.fill_(value)

    def item(self):
        return self.tensor.item()

    def __float__(self):
        return float(self.tensor.item())

    # -- indexing ------------------------------------------------------------
    def __getitem__(self, idx):
        if _is_basic(idx):
            if self._resolver is None:
                return DeviceArray(self._tensor[idx])
            parent = self._resolver
            return DeviceArray(resolver=lambda: parent()[idx])
        return DeviceArray(self.tensor[_to_index(idx, self.device)])

    def __setitem__(self, idx, value):
        t = self.tensor
        if isinstance(value, DeviceArray):
            value = value.tensor
        elif isinstance(value, np.ndarray):
            value = _torch().as_tensor(value, device=t.device, dtype=t.dtype)
        t[_to_index(idx, t.device)] = value

    # -- arithmetic (device) ---------------------------------------------------
    @staticmethod
    def _v(x, like):
        if isinstance(x, DeviceArray):
            return x.tensor
        if isinstance(x, np.ndarray):
            return _torch().as_tensor(x, device=like.device)
        return x

    def _bin(self, other, op):
        t = self.tensor
        return DeviceArray(op(t, self._v(other, t)))

    def __add__(self, o): return self._bin(o, lambda a, b: a + b)
    def __radd__(self, o): return self._bin(o, lambda a, b: b + a)
    def __sub__(self, o): return self._bin(o, lambda a, b: a - b)
    def __rsub__(self, o): return self._bin(o, lambda a, b: b - a)
    def __mul__(self, o): return self._bin(o, lambda a, b: a * b)
    def __rmul__(self, o): return self._bin(o, lambda a, b: b * a)
    def __truediv__(self, o): return self._bin(o, lambda a, b: a / b)
    def __rtruediv__(self, o): return self._bin(o, lambda a, b: b / a)
    def __pow__(self, o): return self._bin(o, lambda a, b: a ** b)
    def __lt__(self, o): return self._bin(o, lambda a, b: a < b)
    def __le__(self, o): return self._bin(o, lambda a, b: a <= b)
    def __gt__(self, o): return self._bin(o, lambda a, b: a > b)
    def __ge__(self, o): return self._bin(o, lambda a, b: a >= b)
    def __neg__(self): return DeviceArray(-self.tensor)
    def __abs__(self): return DeviceArray(self.tensor.abs())

    def _inplace(self, other, op):
        t = self.tensor
        op(t, self._v(other, t))
        return self

    def __iadd__(self, o): return self._inplace(o, lambda a, b: a.add_(b))
    def __isub__(self, o): return self._inplace(o, lambda a, b: a.sub_(b))
    def __imul__(self, o): return self._inplace(o, lambda a, b: a.mul_(b))
    def __itruediv__(self, o): return self._inplace(o, lambda a, b: a.div_(b))

    # -- NumPy protocol: common reductions on the device, the rest via the host ---
    _DEVICE_FUNCS = None

    def __array_function__(self, func, types, args, kwargs):
        torch = _torch()
        table = {
            np.max: lambda a, **k: _red(a, torch.amax, **k),
            np.amax: lambda a, **k: _red(a, torch.amax, **k),
            np.min: lambda a, **k: _red(a, torch.amin, **k),
            np.amin: lambda a, **k: _red(a, torch.amin, **k),
            np.sum: lambda a, **k: _red(a, torch.sum, **k),
            np.mean: lambda a, **k: _red(a, torch.mean, **k),
            np.zeros_like: lambda a, **k: DeviceArray(torch.zeros_like(a.tensor)),
            np.ones_like: lambda a, **k: DeviceArray(torch.ones_like(a.tensor)),
            np.copy: lambda a, **k: a.copy(),
            np.any: lambda a, **k: bool(torch.any(a.tensor).item()),
            np.all: lambda a, **k: bool(torch.all(a.tensor).item()),
            np.shape: lambda a: a.shape,
        }
        fn = table.get(func)
        if fn is not None and isinstance(args[0], DeviceArray):
            return fn(*args, **kwargs)
        conv = [np.asarray(a) if isinstance(a, DeviceArray) else a for a in args]
        return func(*conv, **kwargs)

    def __array_ufunc__(self, ufunc, method, *inputs, **kwargs):
        torch = _torch()
        if method == "__call__" and not kwargs:
            ts = [x.tensor if isinstance(x, DeviceArray) else x for x in inputs]
            unary = {np.abs: torch.abs, np.absolute: torch.abs, np.sqrt: torch.sqrt, np.exp: torch.exp,
                     np.sin: torch.sin, np.cos: torch.cos, np.square: torch.square, np.isfinite: torch.isfinite,
                     np.negative: torch.neg}
            binary = {np.add: torch.add, np.subtract: torch.sub, np.multiply: torch.mul, np.divide: torch.div,
                      np.power: torch.pow, np.maximum: torch.maximum, np.minimum: torch.minimum}
            if ufunc in unary and len(ts) == 1:
                return DeviceArray(unary[ufunc](ts[0]))
            if ufunc in binary and len(ts) == 2:
                a, b = ts
                dev = a.device if hasattr(a, "device") else b.device
                a = a if hasattr(a, "device") else torch.as_tensor(a, device=dev)
                b = b if hasattr(b, "device") else torch.as_tensor(b, device=dev)
                return DeviceArray(binary[ufunc](a, b))
        conv = [np.asarray(x) if isinstance(x, DeviceArray) else x for x in inputs]
        return getattr(ufunc, method)(*conv, **kwargs)


def _red(a, fn, axis=None, **_):
    t = a.tensor
    r = fn(t) if axis is None else fn(t, dim=axis)
    if axis is None:
        return r.item()
    return DeviceArray(r)


# ---------------------------------------------------------------------------
# Backend interface (backends/base.py:14-219)
# ---------------------------------------------------------------------------
class Backend(ABC):
    """Array-provider interface with the reference's method names."""

    @property
    @abstractmethod
    def name(self) -> str: ...

    @property
    @abstractmethod
    def is_gpu(self) -> bool: ...

    def __repr__(self):
        return f"{self.__class__.__name__}(name={self.name}, gpu={self.is_gpu})"


class CudaBackend(Backend):
    """The "cuda" backend (GB300): device arrays + the native FDTD stepper.

    ``precision`` selects the stepper's field type ("fp32" default, "fp64" for
    drop-in checks against the float64 reference)."""

    def __init__(self, device_id: int = 0, precision: str = "fp32"):
        torch = _torch()
        if not torch.cuda.is_available():
            raise ValueError("cuda backend requested but no CUDA device is available")
        if precision not in ("fp32", "fp64"):
            raise ValueError("precision must be 'fp32' or 'fp64'")
        self.device_id = device_id
        self.device = torch.device(f"cuda:{device_id}")
        self.precision = precision
        torch.cuda.set_device(self.device)
        from . import _lib

        _lib.load()  # fail loudly when the native library is missing

    @property
    def name(self) -> str:
        return "cuda"

    @property
    def is_gpu(self) -> bool:
        return True

    @property
    def field_dtype(self):
        torch = _torch()
        return torch.float32 if self.precision == "fp32" else torch.float64

    # dtypes
    @property
    def float32(self): return np.float32
    @property
    def float64(self): return np.float64
    @property
    def complex64(self): return np.complex64
    @property
    def complex128(self): return np.complex128
    @property
    def int32(self): return np.int32
    @property
    def int64(self): return np.int64
    @property
    def pi(self): return math.pi

    # creation
    def zeros(self, shape, dtype=None):
        torch = _torch()
        return DeviceArray(torch.zeros(shape, dtype=_dtype_to_torch(dtype or np.float64), device=self.device))

    def ones(self, shape, dtype=None):
        torch = _torch()
        return DeviceArray(torch.ones(shape, dtype=_dtype_to_torch(dtype or np.float64), device=self.device))

    def empty(self, shape, dtype=None):
        torch = _torch()
        return DeviceArray(torch.empty(shape, dtype=_dtype_to_torch(dtype or np.float64), device=self.device))

    def array(self, data, dtype=None):
        return self.asarray(np.array(np.asarray(data), dtype=dtype) if dtype else np.array(np.asarray(data)))

    def asarray(self, data, dtype=None):
        torch = _torch()
        if isinstance(data, DeviceArray):
            t = data.tensor
            return DeviceArray(t if dtype is None else t.to(_dtype_to_torch(dtype)))
        if isinstance(data, torch.Tensor):
            return DeviceArray(data.to(self.device, dtype=_dtype_to_torch(dtype)))
        arr = np.asarray(data, dtype=dtype)
        return DeviceArray(torch.as_tensor(np.ascontiguousarray(arr), device=self.device))

    def to_numpy(self, array):
        if isinstance(array, DeviceArray):
            return array.to_numpy()
        return np.asarray(array)

    def copy(self, array):
        return array.copy() if isinstance(array, DeviceArray) else self.asarray(np.copy(array))

    # math
    def _t(self, a):
        return self.asarray(a).tensor if not isinstance(a, DeviceArray) else a.tensor

    def sqrt(self, a): return DeviceArray(_torch().sqrt(self._t(a)))
    def exp(self, a): return DeviceArray(_torch().exp(self._t(a)))
    def sin(self, a): return DeviceArray(_torch().sin(self._t(a)))
    def cos(self, a): return DeviceArray(_torch().cos(self._t(a)))
    def abs(self, a): return DeviceArray(_torch().abs(self._t(a)))

    def sum(self, a, axis=None, keepdims=False):
        t = self._t(a)
        return t.sum().item() if axis is None else DeviceArray(t.sum(dim=axis, keepdim=keepdims))

    def max(self, a, axis=None, keepdims=False):
        t = self._t(a)
        return t.max().item() if axis is None else DeviceArray(t.amax(dim=axis, keepdim=keepdims))

    def min(self, a, axis=None, keepdims=False):
        t = self._t(a)
        return t.min().item() if axis is None else DeviceArray(t.amin(dim=axis, keepdim=keepdims))

    def mean(self, a, axis=None, keepdims=False):
        t = self._t(a)
        return t.mean().item() if axis is None else DeviceArray(t.mean(dim=axis, keepdim=keepdims))

    def fft(self, a, axis=-1): return DeviceArray(_torch().fft.fft(self._t(a), dim=axis))
    def ifft(self, a, axis=-1): return DeviceArray(_torch().fft.ifft(self._t(a), dim=axis))
    def fft2(self, a): return DeviceArray(_torch().fft.fft2(self._t(a)))
    def ifft2(self, a): return DeviceArray(_torch().fft.ifft2(self._t(a)))
    def dot(self, a, b): return DeviceArray(_torch().tensordot(self._t(a), self._t(b), dims=1))
    def matmul(self, a, b): return DeviceArray(_torch().matmul(self._t(a), self._t(b)))

    def where(self, cond, x, y):
        torch = _torch()
        c = self._t(cond)
        xx = self._t(x) if isinstance(x, (DeviceArray, np.ndarray)) else torch.as_tensor(x, device=self.device)
        yy = self._t(y) if isinstance(y, (DeviceArray, np.ndarray)) else torch.as_tensor(y, device=self.device)
        return DeviceArray(torch.where(c, xx, yy))

    def synchronize(self):
        _torch().cuda.synchronize(self.device)

    def get_memory_info(self) -> dict:
        torch = _torch()
        free, total = torch.cuda.mem_get_info(self.device)
        return {"free": free, "total": total, "used": total - free,
                "allocated": torch.cuda.memory_allocated(self.device)}


# ---------------------------------------------------------------------------
# registry (backends/backend_manager.py:33-259)
# ---------------------------------------------------------------------------
_CURRENT: Optional[Backend] = None


def list_available_backends() -> list:
    """backend_manager.py:33-67: names usable on this machine."""
    try:
        torch = _torch()
        ok = torch.cuda.is_available()
    except Exception:
        ok = False
    return ["cuda"] if ok else []


def set_backend(backend: str, device_id: int = 0, **kwargs) -> Backend:
    """backend_manager.py:139-186: unknown or unavailable names raise ValueError."""
    global _CURRENT
    name = backend.lower()
    if name == "cuda":
        if "cuda" not in list_available_backends():
            raise ValueError("cuda backend requested but no CUDA device is available")
        _CURRENT = CudaBackend(device_id=device_id, **kwargs)
        return _CURRENT
    raise ValueError(f"Unknown backend '{backend}'. Available backends: {list_available_backends()}")


def get_backend(backend: Optional[str] = None, device_id: int = 0, **kwargs) -> Backend:
    """backend_manager.py:189-241."""
    if backend is not None:
        return set_backend(backend, device_id, **kwargs)
    if _CURRENT is not None:
        return _CURRENT
    if "cuda" in list_available_backends():
        warnings.warn("No backend specified. Auto-selecting the cuda backend.", UserWarning, stacklevel=2)
        return set_backend("cuda", device_id)
    raise ValueError("no backend available: the cuda backend needs a CUDA device")


def get_backend_info() -> dict:
    info = {"available_backends": list_available_backends(), "current_backend": _CURRENT.name if _CURRENT else None}
    try:
        torch = _torch()
        if torch.cuda.is_available():
            info["num_devices"] = torch.cuda.device_count()
            info["cuda_devices"] = [{"id": i, "name": torch.cuda.get_device_name(i),
                                     "compute_capability": torch.cuda.get_device_capability(i)}
                                    for i in range(torch.cuda.device_count())]
    except Exception as e:  # pragma: no cover
        info["cuda_error"] = str(e)
    return info


def resolve(backend) -> Backend:
    if isinstance(backend, Backend):
        return backend
    if isinstance(backend, str):
        return get_backend(backend)
    if backend is None:
        return get_backend()
    # a foreign backend object (e.g. the reference's own) that names itself "cuda"
    if getattr(backend, "name", None) == "cuda" and hasattr(backend, "device"):
        return backend
    raise TypeError("backend must be a Backend instance or string name")
