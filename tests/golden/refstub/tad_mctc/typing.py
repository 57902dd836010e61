"""Type aliases and the ``TensorLike`` base class used by tad-dftd4."""

from __future__ import annotations

from typing import Any, Callable, Literal, TypeAlias, TypedDict, overload  # noqa: F401

import torch

Tensor = torch.Tensor
DD = dict
CNFunc = Callable[..., torch.Tensor]
CountingFunction = Callable[..., torch.Tensor]


class Molecule(TypedDict):
    numbers: torch.Tensor
    positions: torch.Tensor


class TensorLike:
    """Holds a device and a dtype; ``dd`` is the usual keyword dictionary."""

    __slots__ = ("_stub_device", "_stub_dtype")

    def __init__(self, device=None, dtype=None):
        self._stub_device = device if device is not None else torch.device("cpu")
        self._stub_dtype = dtype if dtype is not None else torch.get_default_dtype()

    @property
    def device(self):
        return self._stub_device

    @property
    def dtype(self):
        return self._stub_dtype

    @property
    def dd(self):
        return {"device": self.device, "dtype": self.dtype}
